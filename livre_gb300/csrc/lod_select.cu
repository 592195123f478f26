/*
 * Octree LOD + frustum brick selection on the device.
 *
 * Replaces the recursive CPU traversal of livre/data/DFSTraversal.cpp:29-76
 * driving livre/data/SelectVisibles.cpp:45-131 with a level-synchronous,
 * warp-cooperative traversal: each level is one launch over a device
 * frontier; a node is culled (frustum / clip planes), emitted (LOD visible)
 * or replaced by its 8 children in the next frontier. Emission and child
 * pushes are warp-aggregated (ballot / match + one atomic per group) and
 * compact the output without a separate prefix-sum pass.
 *
 * Bit-exactness: every float operation of a node visit is an explicit IEEE
 * round-to-nearest intrinsic (__fadd_rn, __fmul_rn, __fdiv_rn), in the same
 * order as the reference's FP32 code, so no FMA contraction can change a
 * decision. Per-frame constants (planes, limits, eye) are computed once on
 * the host with the same single-precision formulas.
 */
#include <algorithm>
#include <cmath>

#include "lv_runtime.h"

namespace lv
{
namespace
{
/* ------------------------------------------------------------- host math */
inline float Mh(const float* m, int r, int c) { return m[c * 4 + r]; }

/* 4x4 inverse by Laplace expansion along the first two rows (2x2 minors). */
bool inverse4(const float* m, float* inv)
{
    const float m00 = Mh(m, 0, 0), m01 = Mh(m, 0, 1), m02 = Mh(m, 0, 2),
                m03 = Mh(m, 0, 3);
    const float m10 = Mh(m, 1, 0), m11 = Mh(m, 1, 1), m12 = Mh(m, 1, 2),
                m13 = Mh(m, 1, 3);
    const float m20 = Mh(m, 2, 0), m21 = Mh(m, 2, 1), m22 = Mh(m, 2, 2),
                m23 = Mh(m, 2, 3);
    const float m30 = Mh(m, 3, 0), m31 = Mh(m, 3, 1), m32 = Mh(m, 3, 2),
                m33 = Mh(m, 3, 3);
    const float s0 = m00 * m11 - m10 * m01;
    const float s1 = m00 * m12 - m10 * m02;
    const float s2 = m00 * m13 - m10 * m03;
    const float s3 = m01 * m12 - m11 * m02;
    const float s4 = m01 * m13 - m11 * m03;
    const float s5 = m02 * m13 - m12 * m03;
    const float c5 = m22 * m33 - m32 * m23;
    const float c4 = m21 * m33 - m31 * m23;
    const float c3 = m21 * m32 - m31 * m22;
    const float c2 = m20 * m33 - m30 * m23;
    const float c1 = m20 * m32 - m30 * m22;
    const float c0 = m20 * m31 - m30 * m21;
    const float det =
        s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    if (det == 0.0f || !std::isfinite(det))
        return false;
    const float id = 1.0f / det;
    const float r[4][4] = {
        {(m11 * c5 - m12 * c4 + m13 * c3) * id,
         (-m01 * c5 + m02 * c4 - m03 * c3) * id,
         (m31 * s5 - m32 * s4 + m33 * s3) * id,
         (-m21 * s5 + m22 * s4 - m23 * s3) * id},
        {(-m10 * c5 + m12 * c2 - m13 * c1) * id,
         (m00 * c5 - m02 * c2 + m03 * c1) * id,
         (-m30 * s5 + m32 * s2 - m33 * s1) * id,
         (m20 * s5 - m22 * s2 + m23 * s1) * id},
        {(m10 * c4 - m11 * c2 + m13 * c0) * id,
         (-m00 * c4 + m01 * c2 - m03 * c0) * id,
         (m30 * s4 - m31 * s2 + m33 * s0) * id,
         (-m20 * s4 + m21 * s2 - m23 * s0) * id},
        {(-m10 * c3 + m11 * c1 - m12 * c0) * id,
         (m00 * c3 - m01 * c1 + m02 * c0) * id,
         (-m30 * s3 + m31 * s1 - m32 * s0) * id,
         (m20 * s3 - m21 * s1 + m22 * s0) * id}};
    for (int rr = 0; rr < 4; ++rr)
        for (int cc = 0; cc < 4; ++cc)
            inv[cc * 4 + rr] = r[rr][cc];
    return true;
}

/* ---------------------------------------------------------- device math */
__device__ __forceinline__ float pdot(const float* pl, const float* p)
{
    return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(pl[0], p[0]),
                                         __fmul_rn(pl[1], p[1])),
                               __fmul_rn(pl[2], p[2])),
                     pl[3]);
}

__device__ __forceinline__ bool outside(const float* pl, const float* bmin,
                                        const float* bmax)
{
    float pv[3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
        pv[i] = pl[i] >= 0.0f ? bmax[i] : bmin[i];
    return pdot(pl, pv) < 0.0f;
}

/* 0 = culled, 1 = emit (LOD visible), 2 = descend. SelectVisibles.cpp:66-107 */
__device__ int visit(const LodView& V, uint64_t id)
{
    const uint32_t L = nid_level(id);
    uint32_t bm = V.root_blocks[0] << L;
    bm = max(bm, V.root_blocks[1] << L);
    bm = max(bm, V.root_blocks[2] << L);
    const float denom = __uint2float_rn(bm);
    const uint32_t pos[3] = {nid_x(id), nid_y(id), nid_z(id)};
    float bmin[3], bmax[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
    {
        const float cmin = __fdiv_rn(__int2float_rn(int(pos[a])), denom);
        const float cmax = __fdiv_rn(__int2float_rn(int(pos[a] + 1u)), denom);
        bmin[a] = __fsub_rn(__fmul_rn(cmin, V.world_size[a]), V.half[a]);
        bmax[a] = __fsub_rn(__fmul_rn(cmax, V.world_size[a]), V.half[a]);
    }
#pragma unroll
    for (int p = 0; p < 6; ++p)
        if (outside(V.planes[p], bmin, bmax))
            return 0;
    for (uint32_t c = 0; c < V.n_clip; ++c)
        if (outside(V.clip[c], bmin, bmax))
            return 0;

    const float* np = V.planes[4];
    float vmin[3], vmax[3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
    {
        const bool pos_n = np[i] >= 0.0f;
        vmin[i] = pos_n ? bmin[i] : bmax[i];
        vmax[i] = pos_n ? bmax[i] : bmin[i];
    }
    if (pdot(np, vmin) < 0.0f || pdot(np, vmax) < 0.0f)
    {
#pragma unroll
        for (int i = 0; i < 3; ++i)
            vmin[i] = V.eye_near[i];
    }
    float wspv = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; ++a)
    {
        const float w = __fdiv_rn(__fsub_rn(bmax[a], bmin[a]),
                                  __uint2float_rn(V.block[a]));
        wspv = (a == 0 || w < wspv) ? w : wspv;
    }
    const float ppv = __fdiv_rn(wspv, V.wspp);
    const float dist = fabsf(pdot(np, vmin));
    const float ppvd =
        __fdiv_rn(__fmul_rn(ppv, V.nearp), __fadd_rn(V.nearp, dist));
    bool vis = ppvd <= V.sse;
    vis = (vis && L >= V.min_lod) || L == V.max_lod || L == V.depth - 1u;
    return vis ? 1 : 2;
}

__device__ __forceinline__ uint32_t lanemask_lt()
{
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

/* Zeroes the per-level counters and every view's result words, and writes
 * the level-0 frontier (root blocks in any order). One block per view. */
__global__ void lod_roots_kernel(const LodView* __restrict__ views,
                                 uint32_t n_views, uint64_t* __restrict__ ids,
                                 uint32_t* __restrict__ view_of,
                                 uint32_t* __restrict__ counts,
                                 uint32_t n_counts, uint32_t total_roots,
                                 uint32_t capacity,
                                 const uint32_t* __restrict__ d_total_roots)
{
    /* d_total_roots (nullable): the count in device memory, for launches
     * replayed from a CUDA graph with different views */
    if (d_total_roots)
        total_roots = *d_total_roots;
    const uint32_t v = blockIdx.x;
    if (v == 0)
    {
        for (uint32_t i = threadIdx.x; i < n_counts; i += blockDim.x)
            counts[i] = i == 0 ? min(total_roots, capacity) : 0u;
    }
    if (v >= n_views)
        return;
    const LodView& V = views[v];
    if (threadIdx.x < LV_SELECT_RESULT_WORDS)
        V.result[threadIdx.x] = 0u;
    const uint32_t rx = V.root_blocks[0], ry = V.root_blocks[1],
                   rz = V.root_blocks[2];
    const uint32_t n = rx * ry * rz;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
    {
        const uint32_t x = i / (ry * rz), y = (i / rz) % ry, z = i % rz;
        const uint32_t slot = V.root_offset + i;
        if (slot < capacity)
        {
            ids[slot] = nid_make(0, x, y, z, V.time_step);
            view_of[slot] = v;
        }
    }
}

/* One level of the traversal over frontier items [0, n) strided by the
 * grid: visit, warp-aggregated emission of visible ids per view, 8 child
 * pushes per descending lane. COHERENT: the frontier was written by other
 * CTAs of the same launch, so it is read through L2 (not the SM's L1). */
template <bool COHERENT>
__device__ __forceinline__ void level_items(const LodView* __restrict__ views,
                                            const uint64_t* __restrict__ in_ids,
                                            const uint32_t* __restrict__ in_view, uint32_t n,
                                            uint64_t* __restrict__ out_ids,
                                            uint32_t* __restrict__ out_view,
                                            uint32_t* __restrict__ out_count, uint32_t capacity,
                                            uint32_t* __restrict__ overflow,
                                            bool block_only = false)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt = lanemask_lt();
    const uint32_t first = block_only ? 0u : blockIdx.x * blockDim.x;
    const uint32_t stride = block_only ? blockDim.x : gridDim.x * blockDim.x;
    for (uint32_t base = first; base < n; base += stride)
    {
        const uint32_t i = base + threadIdx.x;
        const bool active = i < n;
        uint64_t id = 0;
        uint32_t v = 0;
        int decision = 0;
        if (active)
        {
            id = COHERENT ? __ldcg(in_ids + i) : in_ids[i];
            v = COHERENT ? __ldcg(in_view + i) : in_view[i];
            decision = visit(views[v], id);
        }
        /* per-view groups of active lanes: visited + emitted counts */
        const uint32_t key = active ? v : 0xFFFFFFFFu;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
        const uint32_t leader = __ffs(peers) - 1u;
        const uint32_t emit_mask = __ballot_sync(0xFFFFFFFFu, decision == 1);
        const uint32_t my_emits = emit_mask & peers;
        uint32_t ebase = 0;
        if (active && lane == leader)
        {
            uint32_t* res = views[v].result;
            atomicAdd(&res[LV_SEL_VISITED], __popc(peers));
            if (my_emits)
            {
                ebase = atomicAdd(&res[LV_SEL_FOUND], __popc(my_emits));
                atomicMax(&res[LV_SEL_MAX_LEVEL], nid_level(id));
            }
        }
        ebase = __shfl_sync(0xFFFFFFFFu, ebase, leader);
        if (decision == 1)
        {
            const uint32_t slot = ebase + __popc(my_emits & lt);
            if (slot < views[v].capacity)
                views[v].out_ids[slot] = id;
        }
        /* children of descending lanes, 8 per lane */
        const uint32_t desc = __ballot_sync(0xFFFFFFFFu, decision == 2);
        uint32_t cbase = 0;
        if (lane == 0 && desc)
            cbase = atomicAdd(out_count, 8u * __popc(desc));
        cbase = __shfl_sync(0xFFFFFFFFu, cbase, 0);
        if (decision == 2)
        {
            const uint32_t slot = cbase + 8u * __popc(desc & lt);
            if (slot + 8u <= capacity)
            {
                const uint32_t L = nid_level(id) + 1u, t = nid_t(id);
                const uint32_t x = nid_x(id) * 2u, y = nid_y(id) * 2u,
                               z = nid_z(id) * 2u;
#pragma unroll
                for (uint32_t c = 0; c < 8; ++c)
                {
                    out_ids[slot + c] =
                        nid_make(L, x + (c >> 2), y + ((c >> 1) & 1u),
                                 z + (c & 1u), t);
                    out_view[slot + c] = v;
                }
            }
            else
                atomicExch(overflow, 1u);
        }
    }
}

__global__ void __launch_bounds__(256)
    lod_level_kernel(const LodView* __restrict__ views,
                     const uint64_t* __restrict__ in_ids,
                     const uint32_t* __restrict__ in_view,
                     const uint32_t* __restrict__ in_count,
                     uint64_t* __restrict__ out_ids,
                     uint32_t* __restrict__ out_view,
                     uint32_t* __restrict__ out_count, uint32_t capacity,
                     uint32_t* __restrict__ overflow)
{
    level_items<false>(views, in_ids, in_view, min(*in_count, capacity), out_ids, out_view,
                       out_count, capacity, overflow);
}

/* WRITTEN = min(FOUND, capacity); OVERFLOW from the frontier flag. */
__global__ void lod_finish_kernel(const LodView* __restrict__ views,
                                  uint32_t n_views,
                                  const uint32_t* __restrict__ overflow)
{
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_views)
        return;
    uint32_t* res = views[v].result;
    res[LV_SEL_WRITTEN] = min(res[LV_SEL_FOUND], views[v].capacity);
    res[LV_SEL_OVERFLOW] = *overflow;
}

/* ---- single-view selection in one cooperative launch ------------------
 * Roots, every level and the result words of one view in one launch whose
 * CTAs are all resident (cooperative launch), separated by a grid barrier
 * instead of a kernel boundary. The view's constants are a kernel
 * parameter. bar[0] counts arrivals, bar[1] is the barrier generation,
 * bar[2] an error flag set when a wait gives up (kSpinLimit polls); the
 * words are zeroed before the launch, with the level counters. */
constexpr uint32_t kSpinLimit = 1u << 22; /* ~0.3 s of 64 ns sleeps */
constexpr uint32_t kSoloItems = 1024;     /* frontier one CTA visits alone */

__device__ __forceinline__ void grid_barrier(uint32_t* bar, uint32_t spin_limit)
{
    __syncthreads();
    if (threadIdx.x == 0)
    {
        volatile uint32_t* gen = bar + 1;
        const uint32_t g = *gen;
        __threadfence();
        if (atomicAdd(bar, 1u) == gridDim.x - 1u)
        {
            atomicExch(bar, 0u);
            __threadfence();
            atomicExch(bar + 1, g + 1u);
        }
        else
        {
            uint32_t polls = 0;
            while (*gen == g)
            {
                if (++polls > spin_limit)
                {
                    atomicExch(bar + 2, 1u); /* gave up: results unusable */
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

__global__ void __launch_bounds__(256)
    lod_fused_kernel(const __grid_constant__ LodView V, uint32_t max_depth,
                     uint64_t* __restrict__ ids0, uint32_t* __restrict__ view0,
                     uint64_t* __restrict__ ids1, uint32_t* __restrict__ view1,
                     uint32_t* __restrict__ counts, uint32_t capacity,
                     uint32_t spin_limit, uint32_t absent_cta)
{
    /* test hook (lv_test_fail_grid_barrier): this CTA never arrives, so the
     * others' bounded waits give up and the result reports it */
    if (blockIdx.x == absent_cta)
        return;
    uint32_t* overflow = counts + kMaxLevels + 1;
    uint32_t* bar = counts + kMaxLevels + 2;
    uint32_t* solo_end = counts + kMaxLevels + 5;
    const LodView* views = &V;
    const uint32_t rx = V.root_blocks[0], ry = V.root_blocks[1], rz = V.root_blocks[2];
    const uint32_t n_roots = min(rx * ry * rz, capacity);
    /* Levels whose frontier is small are visited by CTA 0 alone, separated
     * by block barriers; the other CTAs wait at one grid barrier until the
     * frontier outgrows a CTA (or the selection ends). */
    const bool solo = n_roots <= kSoloItems;
    if (blockIdx.x == 0)
    {
        if (threadIdx.x == 0)
            counts[0] = n_roots;
        if (threadIdx.x < LV_SELECT_RESULT_WORDS)
            V.result[threadIdx.x] = 0u;
    }
    if (!solo || blockIdx.x == 0)
        for (uint32_t i = (solo ? 0u : blockIdx.x * blockDim.x) + threadIdx.x; i < n_roots;
             i += solo ? blockDim.x : gridDim.x * blockDim.x)
        {
            const uint32_t x = i / (ry * rz), y = (i / rz) % ry, z = i % rz;
            ids0[i] = nid_make(0, x, y, z, V.time_step);
            view0[i] = 0u;
        }
    uint32_t l = 0;
    if (solo)
    {
        if (blockIdx.x == 0)
        {
            __syncthreads();
            for (; l < max_depth; ++l)
            {
                const uint32_t n = min(__ldcg(counts + l), capacity);
                if (n == 0 || n > kSoloItems)
                    break; /* the same value in every thread: read after the barrier */
                const bool even = (l & 1u) == 0;
                level_items<true>(views, even ? ids0 : ids1, even ? view0 : view1, n,
                                  even ? ids1 : ids0, even ? view1 : view0, counts + l + 1,
                                  capacity, overflow, true);
                __syncthreads();
            }
            if (threadIdx.x == 0)
                *solo_end = l;
        }
        grid_barrier(bar, spin_limit);
        l = __ldcg(solo_end);
    }
    else
        grid_barrier(bar, spin_limit);
    for (; l < max_depth; ++l)
    {
        const uint32_t n = min(__ldcg(counts + l), capacity);
        if (n == 0 || __ldcg(bar + 2))
            break; /* the same value in every CTA: read after the barrier */
        const bool even = (l & 1u) == 0;
        level_items<true>(views, even ? ids0 : ids1, even ? view0 : view1, n,
                          even ? ids1 : ids0, even ? view1 : view0, counts + l + 1, capacity,
                          overflow);
        grid_barrier(bar, spin_limit);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
        uint32_t* res = V.result;
        res[LV_SEL_WRITTEN] = min(__ldcg(res + LV_SEL_FOUND), V.capacity);
        /* 2: a barrier wait gave up (nothing of the selection is usable) */
        res[LV_SEL_OVERFLOW] = __ldcg(bar + 2) ? 2u : __ldcg(overflow);
    }
}

/* DFS preorder key: root index then the child index (x*4 + y*2 + z) of
 * every level, padded to the tree depth (DFSTraversal.cpp:63-76 visits the
 * roots x, y, z outer to inner and children in NodeId::getChildren order). */
__global__ void dfs_key_kernel(const uint64_t* __restrict__ ids,
                               const uint32_t* __restrict__ result,
                               uint32_t depth, uint32_t rx, uint32_t ry,
                               uint32_t rz, uint64_t* __restrict__ keys,
                               uint64_t* __restrict__ vals, uint32_t n_pad)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad)
        return;
    const uint32_t n = result[LV_SEL_WRITTEN];
    if (i >= n)
    {
        keys[i] = ~0ull;
        vals[i] = ~0ull;
        return;
    }
    const uint64_t id = ids[i];
    const uint32_t L = nid_level(id);
    const uint32_t x = nid_x(id), y = nid_y(id), z = nid_z(id);
    uint64_t key = (uint64_t(x >> L) * ry + (y >> L)) * rz + (z >> L);
    for (uint32_t l = 1; l < depth; ++l)
    {
        uint64_t c = 0;
        if (l <= L)
        {
            const uint32_t s = L - l;
            c = (((x >> s) & 1u) << 2) | (((y >> s) & 1u) << 1) | ((z >> s) & 1u);
        }
        key = key * 8u + c;
    }
    keys[i] = key;
    vals[i] = id;
}

/* One bitonic compare-exchange pass over n_pad (power of two) pairs. */
__global__ void bitonic_pass_kernel(uint64_t* __restrict__ keys,
                                    uint64_t* __restrict__ vals, uint32_t n_pad,
                                    uint32_t j, uint32_t k)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad)
        return;
    const uint32_t p = i ^ j;
    if (p <= i)
        return;
    const bool up = (i & k) == 0;
    const uint64_t a = keys[i], b = keys[p];
    if ((a > b) == up)
    {
        keys[i] = b;
        keys[p] = a;
        const uint64_t t = vals[i];
        vals[i] = vals[p];
        vals[p] = t;
    }
}

/* visitPost (SelectVisibles.cpp:110-131): keep DFS indices [start, end). */
__global__ void slice_kernel(const uint64_t* __restrict__ sorted_ids,
                             uint64_t* __restrict__ out,
                             uint32_t* __restrict__ result, float r0, float r1)
{
    const uint32_t n = result[LV_SEL_WRITTEN];
    const uint32_t start = uint32_t(__fmul_rn(r0, __uint2float_rn(n)));
    const uint32_t end = min(uint32_t(__fmul_rn(r1, __uint2float_rn(n))), n);
    for (uint32_t i = start + threadIdx.x; i < end; i += blockDim.x)
        out[i - start] = sorted_ids[i];
    __syncthreads();
    if (threadIdx.x == 0)
    {
        const uint32_t k = end > start ? end - start : 0u;
        result[LV_SEL_WRITTEN] = k;
        result[LV_SEL_FOUND] = k;
    }
}

} // namespace

void frustum_setup(const float* mv, const float* p, float inv_mv[16],
                   float inv_p[16], float limits[6], float planes[6][4],
                   float eye[3], float dir[3], bool* ok)
{
    *ok = inverse4(mv, inv_mv) && inverse4(p, inv_p);
    if (!*ok)
        return;
    /* vmml::Frustumf(projection): left right bottom top near far */
    const float p22 = Mh(p, 2, 2), p23 = Mh(p, 2, 3);
    const float nearp = p23 / (p22 - 1.0f);
    limits[4] = nearp;
    limits[5] = p23 / (p22 + 1.0f);
    limits[2] = nearp * (Mh(p, 1, 2) - 1.0f) / Mh(p, 1, 1);
    limits[3] = nearp * (Mh(p, 1, 2) + 1.0f) / Mh(p, 1, 1);
    limits[0] = nearp * (Mh(p, 0, 2) - 1.0f) / Mh(p, 0, 0);
    limits[1] = nearp * (Mh(p, 0, 2) + 1.0f) / Mh(p, 0, 0);
    /* FrustumCuller(P * MV): planes from the rows of the clip matrix */
    float row[4][4];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c)
        {
            float acc = 0.0f;
            for (int k = 0; k < 4; ++k)
                acc = acc + Mh(p, r, k) * Mh(mv, k, c);
            row[r][c] = acc;
        }
    for (int c = 0; c < 4; ++c)
    {
        planes[0][c] = row[3][c] + row[0][c];
        planes[1][c] = row[3][c] - row[0][c];
        planes[2][c] = row[3][c] + row[1][c];
        planes[3][c] = row[3][c] - row[1][c];
        planes[4][c] = row[3][c] + row[2][c];
        planes[5][c] = row[3][c] - row[2][c];
    }
    for (int pl = 0; pl < 6; ++pl)
    {
        float* q = planes[pl];
        const float len = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
        const float inv = float(1.0 / double(len));
        for (int c = 0; c < 4; ++c)
            q[c] = q[c] * inv;
    }
    for (int i = 0; i < 3; ++i)
    {
        eye[i] = Mh(inv_mv, i, 3);
        dir[i] = Mh(inv_mv, i, 2);
    }
}

/* The per-view constants of a selection: LV_OK, or a status with the
 * reason in *why. Shared by every selection entry point. */
lv_status fill_lod_view(const lv_volume_info& vol, const lv_camera& cam,
                        const lv_lod_params& p, LodView& V, const char** why)
{
    if (vol.depth == 0 || vol.depth > kMaxLevels)
        return *why = "volume depth out of range", LV_EINVAL;
    if (p.window_height == 0)
        return *why = "window height is 0", LV_EINVAL;
    if (p.n_clip_planes > 6)
        return *why = "more than 6 clip planes", LV_EINVAL;
    float inv_mv[16], inv_p[16], lim[6], planes[6][4], eye[3], dir[3];
    bool ok = false;
    frustum_setup(cam.modelview, cam.projection, inv_mv, inv_p, lim, planes,
                  eye, dir, &ok);
    if (!ok)
        return *why = "singular modelview or projection", LV_EINVAL;
    std::memset(&V, 0, sizeof(V));
    std::memcpy(V.planes, planes, sizeof(planes));
    V.nearp = lim[4];
    for (int i = 0; i < 3; ++i)
        V.eye_near[i] = eye[i] - dir[i] * V.nearp;
    V.wspp = (lim[3] - lim[2]) / float(p.window_height);
    V.sse = p.screen_space_error;
    for (int i = 0; i < 3; ++i)
    {
        V.world_size[i] = vol.world_size[i];
        V.half[i] = vol.world_size[i] * 0.5f;
        V.root_blocks[i] = vol.root_blocks[i];
        if (vol.max_block[i] <= 2u * vol.overlap[i])
            return *why = "max_block <= 2 * overlap", LV_EINVAL;
        V.block[i] = vol.max_block[i] - 2u * vol.overlap[i];
    }
    V.n_clip = p.n_clip_planes;
    std::memcpy(V.clip, p.clip_planes, sizeof(V.clip));
    V.min_lod = p.min_lod;
    V.max_lod = p.max_lod;
    V.depth = vol.depth;
    V.time_step = p.time_step;
    return LV_OK;
}

lv_status make_lod_view(lv_ctx* ctx, const lv_volume_info& vol,
                        const lv_camera& cam, const lv_lod_params& p,
                        LodView& V)
{
    const char* why = "";
    const lv_status st = fill_lod_view(vol, cam, p, V, &why);
    return st == LV_OK ? st : fail(ctx, st, why);
}

uint64_t max_frontier(const lv_volume_info& vol)
{
    const uint64_t roots = uint64_t(vol.root_blocks[0]) * vol.root_blocks[1] *
                           vol.root_blocks[2];
    uint64_t m = roots;
    for (uint32_t l = 1; l < vol.depth; ++l)
        m = std::max(m, roots << (3 * l));
    return m;
}

namespace
{
/* Grid of the cooperative single-view selection on the context's device
 * (0: cooperative launch unavailable). */
uint32_t fused_grid(lv_ctx* ctx)
{
    static std::mutex m;
    static std::vector<int> grids;
    std::lock_guard<std::mutex> lock(m);
    if (grids.size() <= size_t(ctx->device))
        grids.resize(size_t(ctx->device) + 1, -1);
    int& g = grids[size_t(ctx->device)];
    if (g < 0)
    {
        int coop = 0, sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, lod_fused_kernel, 256, 0) !=
            cudaSuccess)
        {
            cudaGetLastError();
            per_sm = 0;
        }
        g = coop && per_sm > 0 ? sms * std::min(per_sm, 2) : 0;
    }
    return uint32_t(g);
}
} // namespace

lv_status scratch_acquire(lv_ctx* ctx, SelectScratch& S, cudaStream_t s)
{
    if (S.free_recorded)
        LV_CUDA(ctx, cudaStreamWaitEvent(s, S.free_event, 0));
    return LV_OK;
}

lv_status scratch_release(lv_ctx* ctx, SelectScratch& S, cudaStream_t s)
{
    if (!S.free_event)
        LV_CUDA(ctx, cudaEventCreateWithFlags(&S.free_event, cudaEventDisableTiming));
    LV_CUDA(ctx, cudaEventRecord(S.free_event, s));
    S.free_recorded = true;
    return LV_OK;
}

uint32_t selection_launches(lv_ctx* ctx, uint32_t n_views, uint32_t depth, bool allow_fused)
{
    return allow_fused && n_views == 1 && fused_grid(ctx) ? 1u : depth + 2u;
}

lv_status run_selection(lv_ctx* ctx, const LodView* host_views,
                        uint32_t n_views, uint32_t max_depth,
                        cudaStream_t stream, bool allow_fused)
{
    SelectScratch& S = ctx->sel;
    if (S.frontier_capacity == 0)
        return fail(ctx, LV_EINVAL, "selection scratch not reserved");
    const uint32_t grid = allow_fused && n_views == 1 ? fused_grid(ctx) : 0u;
    if (grid)
    {
        /* one view: one cooperative launch, its constants a kernel parameter */
        LodView V = host_views[0];
        V.root_offset = 0;
        const uint32_t cap = S.frontier_capacity;
        if (V.root_blocks[0] * V.root_blocks[1] * V.root_blocks[2] > cap)
            return fail(ctx, LV_ENOMEM, "root frontier exceeds scratch capacity");
        uint32_t* counts = S.counts.as<uint32_t>();
        LV_CUDA(ctx, cudaMemsetAsync(counts, 0, sizeof(uint32_t) * (kMaxLevels + 8), stream));
        uint64_t* ids0 = S.ids[0].as<uint64_t>();
        uint64_t* ids1 = S.ids[1].as<uint64_t>();
        uint32_t* view0 = S.view[0].as<uint32_t>();
        uint32_t* view1 = S.view[1].as<uint32_t>();
        /* no level holds more nodes than the octree's widest one: a CTA more
         * than it needs would only add an arrival to each grid barrier */
        uint64_t widest = uint64_t(V.root_blocks[0]) * V.root_blocks[1] * V.root_blocks[2];
        for (uint32_t l = 1; l < max_depth && widest < (uint64_t(1) << 40); ++l)
            widest <<= 3;
        const uint32_t used =
            uint32_t(std::max<uint64_t>(1, std::min<uint64_t>(grid, (widest + 255) / 256)));
        uint32_t spin = kSpinLimit, absent = 0xFFFFFFFFu;
        if (ctx->test_barrier_polls && used > 1)
        {
            spin = ctx->test_barrier_polls;
            absent = used - 1; /* never CTA 0, which writes the result */
            ctx->test_barrier_polls = 0;
        }
        void* args[] = {&V, &max_depth, &ids0, &view0, &ids1, &view1, &counts,
                        const_cast<uint32_t*>(&cap), &spin, &absent};
        LV_CUDA(ctx, cudaLaunchCooperativeKernel(reinterpret_cast<void*>(lod_fused_kernel),
                                                 dim3(used), dim3(256), args, 0, stream));
        return LV_OK;
    }
    LV_CUDA(ctx, S.staging.reserve(sizeof(LodView) * n_views));
    LV_CUDA(ctx, S.views.reserve(sizeof(LodView) * n_views));
    /* The pinned staging copy may still be read by a previous in-flight
     * transfer: wait for the stream before overwriting it. */
    LV_CUDA(ctx, cudaStreamSynchronize(stream));
    std::memcpy(S.staging.ptr, host_views, sizeof(LodView) * n_views);
    uint32_t total_roots = 0;
    for (uint32_t v = 0; v < n_views; ++v)
    {
        S.staging.as<LodView>()[v].root_offset = total_roots;
        total_roots += host_views[v].root_blocks[0] *
                       host_views[v].root_blocks[1] *
                       host_views[v].root_blocks[2];
    }
    LV_CUDA(ctx, cudaMemcpyAsync(S.views.ptr, S.staging.ptr,
                                 sizeof(LodView) * n_views,
                                 cudaMemcpyHostToDevice, stream));
    return enqueue_selection(ctx, S, S.views.as<LodView>(), n_views, total_roots,
                             max_depth, stream);
}

lv_status enqueue_selection(lv_ctx* ctx, SelectScratch& S, const LodView* dviews,
                            uint32_t n_views, uint32_t total_roots, uint32_t max_depth,
                            cudaStream_t stream, const uint32_t* d_total_roots)
{
    const uint32_t cap = S.frontier_capacity;
    if (total_roots > cap)
        return fail(ctx, LV_ENOMEM, "root frontier exceeds scratch capacity");
    uint32_t* counts = S.counts.as<uint32_t>();
    const uint32_t n_counts = kMaxLevels + 2;
    uint32_t* overflow = counts + kMaxLevels + 1;
    lod_roots_kernel<<<n_views, 128, 0, stream>>>(
        dviews, n_views, S.ids[0].as<uint64_t>(), S.view[0].as<uint32_t>(),
        counts, n_counts, total_roots, cap, d_total_roots);
    LV_CUDA(ctx, cudaGetLastError());
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    for (uint32_t l = 0; l < max_depth; ++l)
    {
        const int in = l & 1, out = in ^ 1;
        lod_level_kernel<<<2 * sms, 256, 0, stream>>>(
            dviews, S.ids[in].as<uint64_t>(), S.view[in].as<uint32_t>(),
            counts + l, S.ids[out].as<uint64_t>(), S.view[out].as<uint32_t>(),
            counts + l + 1, cap, overflow);
        LV_CUDA(ctx, cudaGetLastError());
    }
    lod_finish_kernel<<<(n_views + 127) / 128, 128, 0, stream>>>(dviews, n_views,
                                                                 overflow);
    LV_CUDA(ctx, cudaGetLastError());
    return LV_OK;
}

lv_status reserve_frontier(lv_ctx* ctx, SelectScratch& S, uint64_t nodes, cudaStream_t s)
{
    /* grow to powers of two: few reallocations (each one drops the graphs
     * captured on the old queues) */
    uint64_t cap = 64;
    while (cap < nodes && cap < (1u << 24))
        cap <<= 1;
    if (S.frontier_capacity >= cap)
        return LV_OK;
    LV_CUDA(ctx, cudaStreamSynchronize(s));
    if (S.free_recorded) /* the last user may have run on another stream */
        LV_CUDA(ctx, cudaEventSynchronize(S.free_event));
    for (int i = 0; i < 2; ++i)
    {
        LV_CUDA(ctx, S.ids[i].reserve(sizeof(uint64_t) * cap));
        LV_CUDA(ctx, S.view[i].reserve(sizeof(uint32_t) * cap));
    }
    /* level counters, overflow flag, fused-launch barrier words */
    LV_CUDA(ctx, S.counts.reserve(sizeof(uint32_t) * (kMaxLevels + 8)));
    S.frontier_capacity = uint32_t(cap);
    ++S.generation; /* captured graphs referencing the old queues are stale */
    return LV_OK;
}

lv_status range_slice(lv_ctx* ctx, const lv_volume_info& vol,
                      const float range[2], uint64_t* d_ids, uint32_t* d_result,
                      cudaStream_t stream)
{
    uint32_t written = 0;
    LV_CUDA(ctx, cudaMemcpyAsync(&written, d_result + LV_SEL_WRITTEN,
                                 sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                 stream));
    LV_CUDA(ctx, cudaStreamSynchronize(stream));
    uint32_t n_pad = 1;
    while (n_pad < written)
        n_pad <<= 1;
    SelectScratch& S = ctx->sel;
    LV_CUDA(ctx, S.sort.reserve(sizeof(uint64_t) * 2 * n_pad));
    uint64_t* keys = S.sort.as<uint64_t>();
    uint64_t* vals = keys + n_pad;
    const uint32_t tb = 256, nb = (n_pad + tb - 1) / tb;
    dfs_key_kernel<<<nb, tb, 0, stream>>>(d_ids, d_result, vol.depth,
                                          vol.root_blocks[0], vol.root_blocks[1],
                                          vol.root_blocks[2], keys, vals, n_pad);
    for (uint32_t k = 2; k <= n_pad; k <<= 1)
        for (uint32_t j = k >> 1; j > 0; j >>= 1)
            bitonic_pass_kernel<<<nb, tb, 0, stream>>>(keys, vals, n_pad, j, k);
    slice_kernel<<<1, 256, 0, stream>>>(vals, d_ids, d_result, range[0],
                                        range[1]);
    LV_CUDA(ctx, cudaGetLastError());
    return LV_OK;
}

} // namespace lv

extern "C" lv_status lv_select_visible(lv_ctx* ctx, const lv_volume_info* vol,
                                       const lv_camera* camera,
                                       const lv_lod_params* params,
                                       uint64_t* d_out_ids, uint32_t capacity,
                                       uint32_t* d_result, void* stream)
{
    using namespace lv;
    if (!ctx || !vol || !camera || !params || !d_result ||
        (!d_out_ids && capacity))
        return fail(ctx, LV_EINVAL, "null argument");
    std::lock_guard<std::mutex> lock(ctx->mutex);
    LV_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    LodView V;
    lv_status st = make_lod_view(ctx, *vol, *camera, *params, V);
    if (st != LV_OK)
        return st;
    V.out_ids = d_out_ids;
    V.capacity = capacity;
    V.result = d_result;
    st = reserve_frontier(ctx, ctx->sel, max_frontier(*vol), s);
    if (st != LV_OK)
        return st;
    /* the scratch is the renderer's too, whose selection runs on a stream of
     * its own */
    st = scratch_acquire(ctx, ctx->sel, s);
    if (st != LV_OK)
        return st;
    st = run_selection(ctx, &V, 1, vol->depth, s);
    if (st != LV_OK)
        return st;
    const bool full = params->range[0] == 0.0f && params->range[1] == 1.0f;
    if (!full)
    {
        st = range_slice(ctx, *vol, params->range, d_out_ids, d_result, s);
        if (st != LV_OK)
            return st;
    }
    return scratch_release(ctx, ctx->sel, s);
}

extern "C" lv_status lv_select_visible_host(lv_ctx* ctx, const lv_volume_info* vol,
                                            const lv_camera* camera,
                                            const lv_lod_params* params, uint64_t* ids,
                                            uint32_t capacity, uint32_t* result)
{
    using namespace lv;
    if (!ctx || !vol || !camera || !params || !result || (!ids && capacity))
        return fail(ctx, LV_EINVAL, "null argument");
    uint64_t* d_ids = nullptr;
    uint32_t* d_res = nullptr;
    {
        std::lock_guard<std::mutex> lock(ctx->mutex);
        LV_CUDA(ctx, cudaSetDevice(ctx->device));
        const size_t id_bytes = (sizeof(uint64_t) * size_t(capacity) + 255) & ~size_t(255);
        LV_CUDA(ctx, ctx->sel_host_out.reserve(id_bytes + 4 * LV_SELECT_RESULT_WORDS));
        d_ids = ctx->sel_host_out.as<uint64_t>();
        d_res = reinterpret_cast<uint32_t*>(ctx->sel_host_out.as<uint8_t>() + id_bytes);
    }
    /* the legacy default stream: ordered after the context's earlier work on
     * blocking streams, and this call waits for it */
    lv_status st = lv_select_visible(ctx, vol, camera, params, d_ids, capacity, d_res, nullptr);
    if (st != LV_OK)
        return st;
    LV_CUDA(ctx, cudaMemcpy(result, d_res, 4 * LV_SELECT_RESULT_WORDS, cudaMemcpyDeviceToHost));
    const uint32_t n = std::min(result[LV_SEL_WRITTEN], capacity);
    if (n)
        LV_CUDA(ctx, cudaMemcpy(ids, d_ids, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost));
    return LV_OK;
}

/* ------------------------------------------------------------------------
 * LOD selection without any allocation.
 *
 * Some callers cannot allocate device memory when they select bricks: a host
 * application whose caching allocator already owns the GPU's memory (an extra
 * cudaMalloc would fail or fragment it), or a per-frame path where the
 * device-wide synchronisation an allocation may trigger is not acceptable.
 * lv_select_visible_noalloc serves them: its frontier queues live in one
 * fixed device array of this file, so it needs no context and allocates
 * nothing. The caller still passes the output ids and result words.
 *
 * Limits and sharing:
 *  - the array holds kNoAllocFrontier nodes per octree level; a volume whose
 *    largest level has more nodes is rejected with LV_ENOMEM;
 *  - only the full range {0, 1} is supported (the DFS-order range slice needs
 *    sort space); other ranges return LV_EINVAL;
 *  - every call on a device shares the one array, and the array keeps the
 *    last call's contents: the kernels clear what must start at zero
 *    (per-level counters, result words) on every call, but two calls whose
 *    work overlaps on the GPU (different streams, or different host threads
 *    without ordering) race on the array and give wrong results;
 *  - the first call on each device does a one-time set-up: it looks up the
 *    array's device address (cudaGetSymbolAddress, with that device current)
 *    and the SM count, and caches both; make that first call before any
 *    stream capture on the device;
 *  - the array is device memory of this file's module: with CUDA's lazy
 *    module loading it is reserved when the module first loads on a device
 *    (this call's set-up, or any selection of lv_render / lv_select_visible),
 *    so make that first use before the application's allocator takes the
 *    GPU's memory;
 *  - the per-view constants reach the device as a kernel parameter (a
 *    one-thread store into the array), so no host buffer outlives the call.
 * ---------------------------------------------------------------------- */
namespace lv
{
namespace
{
constexpr uint32_t kNoAllocFrontier = 262144; /* nodes per octree level */
constexpr uint32_t kNoAllocMaxDevices = 64;
constexpr uint64_t kNoAllocIds = 0;                                   /* 2 x u64 queues */
constexpr uint64_t kNoAllocViews = kNoAllocIds + 16ull * kNoAllocFrontier; /* 2 x u32 */
constexpr uint64_t kNoAllocCounts = kNoAllocViews + 8ull * kNoAllocFrontier;
constexpr uint64_t kNoAllocLod = kNoAllocCounts + 256;
constexpr uint64_t kNoAllocBytes = kNoAllocLod + ((sizeof(LodView) + 255) & ~size_t(255));

/* 24 B per frontier node + counters + one LodView: about 6.3 MB per device. */
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mutex;
unsigned char* g_noalloc_ptr[kNoAllocMaxDevices] = {};
int g_noalloc_sms[kNoAllocMaxDevices] = {};

/* Device address of g_noalloc_scratch on `dev` (the current device) and the
 * device's SM count, looked up once per device. */
lv_status noalloc_scratch(int dev, unsigned char** out, int* sms)
{
    if (dev < 0 || dev >= int(kNoAllocMaxDevices))
        return LV_EDEVICE;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev])
    {
        void* p = nullptr;
        int n = 0;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p ||
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            n <= 0)
        {
            cudaGetLastError(); /* this call's own error: none was pending on entry */
            return LV_EDEVICE;
        }
        g_noalloc_sms[dev] = n;
        g_noalloc_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_noalloc_ptr[dev];
    *sms = g_noalloc_sms[dev];
    return LV_OK;
}

/* A launch of this call failed: its error, cleared. */
lv_status launched()
{
    return cudaGetLastError() == cudaSuccess ? LV_OK : LV_EDEVICE;
}

/* Stores a selection's per-view constants, passed by value, at `dst`:
 * the view reaches the device as a kernel parameter, not as a copy of
 * host memory. */
__global__ void lod_view_store_kernel(const __grid_constant__ LodView V, LodView* dst)
{
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&V);
    uint32_t* d = reinterpret_cast<uint32_t*>(dst);
    for (uint32_t i = threadIdx.x; i < sizeof(LodView) / 4; i += blockDim.x)
        d[i] = src[i];
}
} // namespace
} // namespace lv

extern "C" lv_status lv_select_visible_noalloc(const lv_volume_info* vol,
                                               const lv_camera* camera,
                                               const lv_lod_params* params,
                                               uint64_t* d_out_ids, uint32_t capacity,
                                               uint32_t* d_result, void* stream)
{
    using namespace lv;
    if (!vol || !camera || !params || !d_result || (!d_out_ids && capacity))
        return LV_EINVAL;
    if (!(params->range[0] == 0.0f && params->range[1] == 1.0f))
        return LV_EINVAL;
    if (vol->depth == 0 || vol->depth > kMaxLevels)
        return LV_EINVAL;
    if (max_frontier(*vol) > kNoAllocFrontier)
        return LV_ENOMEM; /* the octree needs more than the fixed scratch holds */
    /* an error left by the caller's earlier work is not this call's: report
     * it without clearing it */
    if (cudaPeekAtLastError() != cudaSuccess)
        return LV_EDEVICE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
    {
        cudaGetLastError();
        return LV_EDEVICE;
    }
    unsigned char* base = nullptr;
    int sms = 0;
    lv_status st = noalloc_scratch(dev, &base, &sms);
    if (st != LV_OK)
        return st;
    LodView V;
    const char* why = "";
    st = fill_lod_view(*vol, *camera, *params, V, &why);
    if (st != LV_OK)
        return st;
    V.out_ids = d_out_ids;
    V.capacity = capacity;
    V.result = d_result;
    V.root_offset = 0;
    const uint32_t roots = vol->root_blocks[0] * vol->root_blocks[1] * vol->root_blocks[2];
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    LodView* dview = reinterpret_cast<LodView*>(base + kNoAllocLod);
    uint64_t* ids[2] = {reinterpret_cast<uint64_t*>(base + kNoAllocIds),
                        reinterpret_cast<uint64_t*>(base + kNoAllocIds) + kNoAllocFrontier};
    uint32_t* views[2] = {reinterpret_cast<uint32_t*>(base + kNoAllocViews),
                          reinterpret_cast<uint32_t*>(base + kNoAllocViews) + kNoAllocFrontier};
    uint32_t* counts = reinterpret_cast<uint32_t*>(base + kNoAllocCounts);
    uint32_t* overflow = counts + kMaxLevels + 1;
    lod_view_store_kernel<<<1, 128, 0, s>>>(V, dview);
    if ((st = launched()) != LV_OK)
        return st;
    lod_roots_kernel<<<1, 128, 0, s>>>(dview, 1, ids[0], views[0], counts, kMaxLevels + 2,
                                       roots, kNoAllocFrontier, nullptr);
    if ((st = launched()) != LV_OK)
        return st;
    for (uint32_t l = 0; l < vol->depth; ++l)
    {
        const int in = l & 1, out = in ^ 1;
        lod_level_kernel<<<2 * sms, 256, 0, s>>>(dview, ids[in], views[in], counts + l,
                                                 ids[out], views[out], counts + l + 1,
                                                 kNoAllocFrontier, overflow);
        if ((st = launched()) != LV_OK)
            return st;
    }
    lod_finish_kernel<<<1, 128, 0, s>>>(dview, 1, overflow);
    return launched();
}

extern "C" lv_status lv_test_fail_grid_barrier(lv_ctx* ctx, uint32_t polls)
{
    using namespace lv;
    if (!ctx || polls == 0 || polls > kSpinLimit)
        return fail(ctx, LV_EINVAL, "polls must be in [1, 2^22]");
    std::lock_guard<std::mutex> lock(ctx->mutex);
    ctx->test_barrier_polls = polls;
    return LV_OK;
}
