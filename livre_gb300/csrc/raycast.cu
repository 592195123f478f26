/*
 * Residency resolve, leaf-grid build and the ray-cast kernel.
 *
 * Replaces the per-brick GL draw loop of livre/eq/render/RayCastRenderer.cpp
 * (onFrameRender :467-481, renderBrick :503-571) and the fragment shader
 * livre/eq/render/shaders/fragRayCast.glsl:113-207. Instead of one draw call
 * per brick with a read-modify-write of an RGBA32F image, one thread walks one
 * ray through every brick in ray order:
 *
 *  - the rendering set (visible bricks, or their nearest resident ancestors,
 *    RenderingSetGeneratorFilter.cpp:32-111) is splatted into a dense leaf
 *    grid at the finest octree level: one 32-bit entry per finest cell,
 *    (level << 27 | pool slot), coarser level winning;
 *  - samples lie on the global grid t = tnearGlobal + k * step, exactly the
 *    positions the shader's residue snapping produces (fragRayCast.glsl:
 *    142-147); a sample belongs to the brick whose cell contains it;
 *  - voxels are read straight from the HBM brick pool (nearest or trilinear,
 *    clamp to edge), mapped through the 1D transfer function (linear,
 *    clamp to edge) and composited front to back with the shader's opacity
 *    correction 1 - (1 - min(a, 255/256))^(32 / nSamples) and early exit.
 *
 * Ray geometry (direction, box and near-plane distances, sample positions,
 * cell and voxel coordinates) uses explicit IEEE round-to-nearest float
 * intrinsics in a fixed order, so every sample reads the same voxels as the
 * CPU oracle; shading runs in FP32 with fused multiply-adds.
 */
#include <algorithm>
#include <cmath>

#include "lv_runtime.h"

namespace lv
{
namespace
{
/* std::min / std::max semantics (first argument on ties), as the oracle. */
__device__ __forceinline__ float smin(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float smax(float a, float b) { return a < b ? b : a; }

/* Emits (id, slot) into the rendering set of the view. */
__device__ __forceinline__ void emit_render(const ResolveView& R, uint64_t id,
                                            uint32_t slot)
{
    const uint32_t k = atomicAdd(&R.counters[FC_RENDERED], 1u);
    if (k < R.render_capacity)
    {
        R.render_ids[k] = id;
        R.render_slots[k] = slot;
    }
    else
        atomicExch(&R.counters[FC_ERROR], 1u);
}

/* For each visible id: resident -> rendering set; missing -> missing list
 * and (async mode) the nearest resident ancestor, once per view. */
__device__ void resolve_body(const ResolveView& R, uint32_t first, uint32_t stride)
{
    const uint32_t n = *R.n_visible_ptr;
    for (uint32_t i = first; i < n; i += stride)
    {
        const uint64_t id = R.visible[i];
        const uint32_t L = nid_level(id);
        if (L >= R.depth || nid_x(id) >= (R.root_blocks[0] << L) ||
            nid_y(id) >= (R.root_blocks[1] << L) || nid_z(id) >= (R.root_blocks[2] << L))
        {
            atomicExch(&R.counters[FC_ERROR], 2u); /* id outside this octree */
            continue;
        }
        const uint64_t idx = node_index(R.level_offset, R.root_blocks, id);
        if (idx >= R.n_nodes)
        {
            atomicExch(&R.counters[FC_ERROR], 2u);
            continue;
        }
        const int32_t slot = R.node_table[idx];
        if (slot >= 0)
        {
            R.node_stamp[idx] = R.frame;
            R.view_stamp[idx] = R.view_frame;
            atomicAdd(&R.counters[FC_AVAILABLE], 1u);
            emit_render(R, id, uint32_t(slot));
            if (R.synchronous)
            {
                /* no ancestor fallback: the rendering set is part of the
                 * visible cut, nothing to prune */
                atomicAdd(&R.counters[FC_KEPT], 1u);
                atomicMax(&R.counters[FC_MAX_LEVEL], L + 1u);
            }
            continue;
        }
        atomicAdd(&R.counters[FC_NOT_AVAILABLE], 1u);
        const uint32_t m = atomicAdd(&R.counters[FC_MISSING], 1u);
        if (m < R.missing_capacity)
            R.missing[m] = id;
        if (R.synchronous)
            continue;
        uint64_t cur = id;
        while (nid_level(cur) > 0)
        {
            const uint32_t L = nid_level(cur) - 1u;
            cur = nid_make(L, nid_x(cur) >> 1, nid_y(cur) >> 1, nid_z(cur) >> 1,
                           nid_t(cur));
            const uint64_t pidx = node_index(R.level_offset, R.root_blocks, cur);
            const int32_t ps = R.node_table[pidx];
            if (ps >= 0)
            {
                /* the exchange comes first: on the single-view path the view
                 * stamps and the in-use stamps are the same array */
                if (atomicExch(&R.view_stamp[pidx], R.view_frame) != R.view_frame)
                    emit_render(R, cur, uint32_t(ps));
                R.node_stamp[pidx] = R.frame;
                break;
            }
        }
    }
}

/* Drops rendering-set entries that have an ancestor in the set, as
 * RenderingSetGenerator::generateRenderingSet does (RenderingSetGeneratorFilter
 * .cpp:63-79): every entry of this view carries view_stamp == view_frame. */
__device__ void prune_body(const ResolveView& R, uint32_t first, uint32_t stride)
{
    const uint32_t n = min(R.counters[FC_RENDERED], R.render_capacity);
    for (uint32_t e = first; e < n; e += stride)
    {
        const uint64_t id = R.render_ids[e];
        uint64_t cur = id;
        bool shadowed = false;
        while (nid_level(cur) > 0)
        {
            cur = nid_make(nid_level(cur) - 1u, nid_x(cur) >> 1, nid_y(cur) >> 1,
                           nid_z(cur) >> 1, nid_t(cur));
            if (R.view_stamp[node_index(R.level_offset, R.root_blocks, cur)] == R.view_frame)
            {
                shadowed = true;
                break;
            }
        }
        if (shadowed)
            R.render_ids[e] = kInvalidNode;
        else
        {
            atomicAdd(&R.counters[FC_KEPT], 1u);
            atomicMax(&R.counters[FC_MAX_LEVEL], nid_level(id) + 1u);
        }
    }
}

/* Splats the rendering set into the leaf grid; one warp per entry. */
__device__ void leaf_fill_body(const ResolveView& R, uint32_t warp, uint32_t nwarps)
{
    const uint32_t n = min(R.counters[FC_RENDERED], R.render_capacity);
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t e = warp; e < n; e += nwarps)
    {
        const uint64_t id = R.render_ids[e];
        if (id == kInvalidNode)
            continue;
        const uint32_t slot = R.render_slots[e];
        const uint32_t L = nid_level(id);
        const uint32_t sh = R.Lf - L;
        const uint32_t side = 1u << sh;
        const uint32_t x0 = nid_x(id) << sh, y0 = nid_y(id) << sh,
                       z0 = nid_z(id) << sh;
        const uint32_t key = (L << kLeafSlotBits) | (slot & kLeafSlotMask);
        const uint64_t cells = uint64_t(side) * side * side;
        for (uint64_t c = lane; c < cells; c += 32)
        {
            const uint32_t cx = x0 + uint32_t(c % side);
            const uint32_t cy = y0 + uint32_t((c / side) % side);
            const uint32_t cz = z0 + uint32_t(c / (uint64_t(side) * side));
            if (cx < R.dims[0] && cy < R.dims[1] && cz < R.dims[2])
                atomicMin(&R.leaf[(uint64_t(cz) * R.dims[1] + cy) * R.dims[0] + cx],
                          key);
        }
    }
}

__global__ void resolve_kernel(ResolveView R)
{
    resolve_body(R, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}
__global__ void prune_kernel(ResolveView R)
{
    prune_body(R, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}
__global__ void leaf_fill_kernel(ResolveView R)
{
    leaf_fill_body(R, (blockIdx.x * blockDim.x + threadIdx.x) >> 5,
                   (gridDim.x * blockDim.x) >> 5);
}
/* multi-view variants: blockIdx.y selects the view */
__global__ void resolve_views_kernel(const ResolveView* __restrict__ Rs)
{
    resolve_body(Rs[blockIdx.y], blockIdx.x * blockDim.x + threadIdx.x,
                 gridDim.x * blockDim.x);
}
__global__ void prune_views_kernel(const ResolveView* __restrict__ Rs)
{
    prune_body(Rs[blockIdx.y], blockIdx.x * blockDim.x + threadIdx.x,
               gridDim.x * blockDim.x);
}
__global__ void leaf_fill_views_kernel(const ResolveView* __restrict__ Rs)
{
    leaf_fill_body(Rs[blockIdx.y], (blockIdx.x * blockDim.x + threadIdx.x) >> 5,
                   (gridDim.x * blockDim.x) >> 5);
}

/* nSamplesPerRay from the finest rendered level (RayCastRenderer.cpp:
 * 216-233 for LV_STEP_REFERENCE; half a voxel for LV_STEP_HALF_VOXEL). */
__device__ void step_body(uint32_t* counters, uint32_t fixed, uint32_t policy,
                          uint32_t max_voxel_dim, uint32_t depth)
{
    uint32_t n = fixed;
    if (n == 0)
    {
        const uint32_t ml = counters[FC_MAX_LEVEL];
        const uint32_t L = ml ? ml - 1u : 0u;
        const uint32_t shift = depth - L - 1u;
        if (policy == LV_STEP_HALF_VOXEL)
            n = (2u * max_voxel_dim) >> shift;
        else
        {
            const float at_lod = float(max_voxel_dim) / float(1u << shift);
            n = uint32_t(fmaxf(at_lod, 512.0f));
        }
        if (n == 0)
            n = 1;
    }
    counters[FC_SAMPLES_PER_RAY] = n;
}

/* nSamplesPerRay of a view from its finest rendered level (the rule of
 * step_body); every ray-cast CTA of lv_render evaluates it, the first one
 * also stores it for the frame statistics. */
__device__ __forceinline__ uint32_t view_samples(const RayView& V)
{
    uint32_t n = V.samples_fixed;
    if (n == 0)
    {
        const uint32_t ml = V.counters[FC_MAX_LEVEL];
        const uint32_t L = ml ? ml - 1u : 0u;
        const uint32_t shift = V.depth - L - 1u;
        if (V.step_policy == LV_STEP_HALF_VOXEL)
            n = (2u * V.max_voxel_dim) >> shift;
        else
            n = uint32_t(fmaxf(float(V.max_voxel_dim) / float(1u << shift), 512.0f));
        if (n == 0)
            n = 1;
    }
    return n;
}

__device__ __forceinline__ uint32_t frame_samples(const RayView& V)
{
    const uint32_t n = view_samples(V);
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0)
        V.counters[FC_SAMPLES_PER_RAY] = n;
    return n;
}

__global__ void step_views_kernel(const RayView* __restrict__ views, uint32_t n)
{
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n)
        step_body(views[v].counters, views[v].samples_fixed, views[v].step_policy,
                  views[v].max_voxel_dim, views[v].depth);
}

/* Hardware base-2 exponential / logarithm (PTX ex2/lg2, approximate, FTZ). */
__device__ __forceinline__ float ex2_approx(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float lg2_approx(float x)
{
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ unsigned long long globaltimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

/* One voxel as a float (the GL shader's conversion of an unsigned, signed or
 * float texel, fragRayCast.glsl:179-197; RayCastRenderer.cpp:236-277). DT is
 * the voxel type, or kDtAny for a type chosen at run time by `dt`. */
template <int DT>
__device__ __forceinline__ float ldv(const uint8_t* p, uint32_t dt)
{
    if (DT == LV_DT_UINT16)
        return float(__ldg(reinterpret_cast<const uint16_t*>(p)));
    if (DT == LV_DT_UINT8)
        return float(__ldg(p));
    switch (dt)
    {
    case LV_DT_INT8: return float(__ldg(reinterpret_cast<const signed char*>(p)));
    case LV_DT_INT16: return float(__ldg(reinterpret_cast<const short*>(p)));
    case LV_DT_UINT32: return __uint2float_rn(__ldg(reinterpret_cast<const unsigned int*>(p)));
    case LV_DT_INT32: return __int2float_rn(__ldg(reinterpret_cast<const int*>(p)));
    case LV_DT_FLOAT: return __ldg(reinterpret_cast<const float*>(p));
    case LV_DT_UINT16: return float(__ldg(reinterpret_cast<const uint16_t*>(p)));
    default: return float(__ldg(p));
    }
}

/* One voxel as a float, read only when `on` (else 0). For uint8 and uint16
 * the load itself is predicated (inline PTX), so a masked sample of the
 * look-ahead march costs no branch and touches no memory; the other types
 * branch. */
template <int DT>
__device__ __forceinline__ float ldv_masked(const uint8_t* p, uint32_t dt, bool on)
{
    if (DT == LV_DT_UINT8)
    {
        uint32_t v = 0;
        asm("{\n\t.reg .pred q;\n\t.reg .u64 g;\n\tcvta.to.global.u64 g, %1;\n\t"
            "setp.ne.b32 q, %2, 0;\n\t@q ld.global.nc.u8 %0, [g];\n\t}"
            : "+r"(v)
            : "l"(p), "r"(uint32_t(on)));
        return float(v);
    }
    if (DT == LV_DT_UINT16)
    {
        uint32_t v = 0;
        asm("{\n\t.reg .pred q;\n\t.reg .u64 g;\n\tcvta.to.global.u64 g, %1;\n\t"
            "setp.ne.b32 q, %2, 0;\n\t@q ld.global.nc.u16 %0, [g];\n\t}"
            : "+r"(v)
            : "l"(p), "r"(uint32_t(on)));
        return float(v);
    }
    return on ? ldv<DT>(p, dt) : 0.0f;
}

/* The two voxel quads of a trilinear sample in a uint8 quad-layout brick
 * (quad_layout: voxels (x, y), (x + 1, y), (x, y + 1), (x + 1, y + 1) in
 * bytes 0 to 3), slices z and z + 1 at byte offsets 0 and dz from p, read
 * only when `on` under one predicate; when !on the registers hold whatever
 * they held (any byte converts to a finite float, and the sample is
 * masked). */
__device__ __forceinline__ void ld_quads2(const uint8_t* p, uint32_t dz, bool on,
                                          uint32_t (&q)[2])
{
    asm("{\n\t.reg .pred q;\n\t.reg .u64 g, h;\n\tcvta.to.global.u64 g, %2;\n\t"
        "cvt.u64.u32 h, %4;\n\tadd.u64 h, g, h;\n\t"
        "setp.ne.b32 q, %3, 0;\n\t"
        "@q ld.global.nc.u32 %0, [g];\n\t"
        "@q ld.global.nc.u32 %1, [h];\n\t}"
        : "=r"(q[0]), "=r"(q[1])
        : "l"(p), "r"(uint32_t(on)), "r"(dz));
}

/* The same with the slice pitch DZ an immediate offset (fixed-pitch
 * kernels). */
template <int DZ>
__device__ __forceinline__ void ld_quads2(const uint8_t* p, bool on, uint32_t (&q)[2])
{
    asm("{\n\t.reg .pred q;\n\t.reg .u64 g;\n\tcvta.to.global.u64 g, %2;\n\t"
        "setp.ne.b32 q, %3, 0;\n\t"
        "@q ld.global.nc.u32 %0, [g];\n\t"
        "@q ld.global.nc.u32 %1, [g+%4];\n\t}"
        : "=r"(q[0]), "=r"(q[1])
        : "l"(p), "r"(uint32_t(on)), "n"(DZ));
}

/* The voxels a sample reads and its interpolation weights; loaded one
 * sample ahead of the compositing (march) so that the loads of the next
 * sample are in flight while the current one is composited. The trilinear
 * taps of the fixed-pitch voxel-quad kernels (raw_taps) stay as the two
 * loaded quad words until the sample is composited: two registers per tap
 * set instead of eight. */
template <int FILTER>
struct Taps
{
    static constexpr int N = FILTER == LV_FILTER_TRILINEAR ? 8 : 1;
    float c[N];
    uint32_t q[2]; /* raw_taps: the quads of slices z and z + 1 */
    float fx, fy, fz;
};

template <int DT, int FILTER, int EDGE>
__host__ __device__ constexpr bool raw_taps()
{
    return DT == LV_DT_UINT8 && FILTER == LV_FILTER_TRILINEAR &&
           quad_layout(DT, EDGE > 1 ? EDGE : 0);
}

/* The view constants the per-sample steps read (the transfer function and
 * its coordinate map, the early-termination opacity, the last trilinear
 * base voxel). A kernel that renders one view passes its RayView parameter
 * itself (constant-bank operands); the persistent batch kernel, whose view
 * changes from tile to tile, passes this register copy instead of reading
 * its shared-memory view on every sample. */
struct HotView
{
    const float4* tf;
    float tf_mul, tf_add, tf_last, early;
    uint32_t max_base;
};

__device__ __forceinline__ HotView hot_view(const RayView& V)
{
    HotView h;
    h.tf = V.tf;
    h.tf_mul = V.tf_mul;
    h.tf_add = V.tf_add;
    h.tf_last = V.tf_last;
    h.early = V.early;
    h.max_base = V.max_base;
    return h;
}

/* Voxels around slot coordinate s (nearest: s = local position; trilinear:
 * s = local position - 0.5, texel centres on integers). EDGE = 1 clamps every
 * tap to the brick (GL_CLAMP_TO_EDGE, needed without overlap); EDGE = 0 uses
 * one base address and offsets to the other taps, valid when every overlap
 * >= 1; EDGE = n > 1 is EDGE = 0 for bricks of n x n voxels in x and y (the
 * row and slice pitches become immediate offsets of one pointer). */
template <int DT, int FILTER, int EDGE, class HV>
__device__ __forceinline__ void load_taps(const RayView& V, const HV& H, const uint8_t* brick,
                                          const float s[3], Taps<FILTER>& T, bool on)
{
    /* the voxels are read only when `on` (the sample has data) */
    auto ld = [&](const uint8_t* q) { return ldv_masked<DT>(q, V.dtype, on); };
    constexpr int NX = EDGE > 1 ? EDGE : 0;
    /* voxel quads (quad_layout): known from the pitch for fixed-pitch
     * kernels, else the view's flag */
    const bool quads = DT == LV_DT_UINT8 && (NX ? quad_layout(DT, NX) : V.quads != 0);
    /* bytes per stored voxel element */
    const int bpv = DT == LV_DT_UINT16 ? 2 : DT == LV_DT_UINT8 ? (quads ? 4 : 1) : int(V.bpv);
    const int n0 = NX ? NX : int(V.N[0]), n1 = NX ? NX : int(V.N[1]), n2 = int(V.N[2]);
    if (FILTER == LV_FILTER_NEAREST)
    {
        const int x = min(max(int(floorf(s[0])), 0), n0 - 1);
        const int y = min(max(int(floorf(s[1])), 0), n1 - 1);
        const int z = min(max(int(floorf(s[2])), 0), n2 - 1);
        T.c[0] = ld(brick + ((z * n1 + y) * n0 + x) * bpv);
        return;
    }
    /* floor by adding 2^23 rounding down (exact for |s| < 2^22), no
     * conversion instruction; x and y as one packed pair */
    const float2 kM = make_float2(8388608.0f, 8388608.0f);
    const float2 sxy = make_float2(s[0], s[1]);
    const float2 fxy0 = __fadd2_rn(__fadd2_rd(sxy, kM), make_float2(-8388608.0f, -8388608.0f));
    const float fx0 = fxy0.x, fy0 = fxy0.y;
    const float fz0 = __fadd_rd(s[2], 8388608.0f) - 8388608.0f;
    const float2 fxy = __ffma2_rn(fxy0, make_float2(-1.0f, -1.0f), sxy); /* s - floor(s) */
    T.fx = fxy.x;
    T.fy = fxy.y;
    T.fz = s[2] - fz0;
    const int ix = int(fx0), iy = int(fy0), iz = int(fz0);
    if (EDGE == 1)
    {
        const int x0 = min(max(ix, 0), n0 - 1), x1 = min(max(ix + 1, 0), n0 - 1);
        const int y0 = min(max(iy, 0), n1 - 1), y1 = min(max(iy + 1, 0), n1 - 1);
        const int z0 = min(max(iz, 0), n2 - 1), z1 = min(max(iz + 1, 0), n2 - 1);
        const int r00 = (z0 * n1 + y0) * n0, r01 = (z0 * n1 + y1) * n0;
        const int r10 = (z1 * n1 + y0) * n0, r11 = (z1 * n1 + y1) * n0;
        T.c[0] = ld(brick + (r00 + x0) * bpv);
        T.c[1] = ld(brick + (r00 + x1) * bpv);
        T.c[2] = ld(brick + (r01 + x0) * bpv);
        T.c[3] = ld(brick + (r01 + x1) * bpv);
        T.c[4] = ld(brick + (r10 + x0) * bpv);
        T.c[5] = ld(brick + (r10 + x1) * bpv);
        T.c[6] = ld(brick + (r11 + x0) * bpv);
        T.c[7] = ld(brick + (r11 + x1) * bpv);
    }
    else
    {
        /* every overlap >= 1: for a sample in cell c the slot coordinate is in
         * [O - 1/2, O + B - 1/2], so the base voxel is in [0, N - 2] on each
         * axis and all eight taps are in the slot. One unsigned clamp of the
         * linear base keeps any tap inside the slot whatever the inputs. */
        const uint32_t base =
            min(__float2uint_rz(fmaf(fmaf(fz0, float(n1), fy0), float(n0), fx0)), H.max_base);
        const int dy = n0 * bpv, dz = n0 * n1 * bpv;
        const uint8_t* p00 = brick + base * bpv;
        const uint8_t* p01 = p00 + dy;
        const uint8_t* p10 = p00 + dz;
        const uint8_t* p11 = p10 + dy;
        if (raw_taps<DT, FILTER, EDGE>())
        {
            /* the quads of slices z and z + 1, kept raw until the sample is
             * composited. The address is formed as a 64-bit product: the same
             * address as p00's 32-bit one compiled to a schedule that ray
             * casts the 2048^3 / 1080p orbit 11 % slower (0.259 against
             * 0.232 ms). */
            ld_quads2<4 * NX * NX>(brick + uint64_t(base) * 4u, on, T.q);
            return;
        }
        if (DT == LV_DT_UINT8 && quads)
        {
            /* the quad layout in a generic-pitch kernel: two quad loads,
             * converted here */
            uint32_t q[2];
            ld_quads2(p00, uint32_t(dz), on, q);
#pragma unroll
            for (int k = 0; k < 4; ++k)
            {
                T.c[k] = float((q[0] >> (8 * k)) & 0xFFu);
                T.c[4 + k] = float((q[1] >> (8 * k)) & 0xFFu);
            }
            return;
        }
        T.c[0] = ld(p00);
        T.c[1] = ld(p00 + bpv);
        T.c[2] = ld(p01);
        T.c[3] = ld(p01 + bpv);
        T.c[4] = ld(p10);
        T.c[5] = ld(p10 + bpv);
        T.c[6] = ld(p11);
        T.c[7] = ld(p11 + bpv);
    }
}

/* Trilinear weights applied x, then y, then z (the oracle's order):
 *   a0 = lerp(c0, c1, fx)  a1 = lerp(c2, c3, fx)  a2 = lerp(c4, c5, fx)
 *   a3 = lerp(c6, c7, fx)  b0 = lerp(a0, a1, fy)  b1 = lerp(a2, a3, fy)
 *   v  = lerp(b0, b1, fz), lerp(a, b, f) = fma(b - a, f, a).
 * Independent lerps run as pairs in packed FP32 instructions (FFMA2: one
 * issue for two IEEE fused multiply-adds, each rounded as the scalar one;
 * b - a as fma(a, -1, b) is the same single rounding), paired so that every
 * result lands in the register pair the next stage reads: (a0, a2) and
 * (a1, a3), then (b0, b1). */
template <int FILTER, bool RAW>
__device__ __forceinline__ float interp(const Taps<FILTER>& T)
{
    if (FILTER == LV_FILTER_NEAREST)
        return T.c[0];
    const float2 m1 = make_float2(-1.0f, -1.0f);
    const float2 fx = make_float2(T.fx, T.fx);
    float2 a02, a13;
    if (RAW)
    {
        /* a voxel byte b placed by a byte permute into the mantissa of 2^23
         * is the float 2^23 + b (exact, no conversion instruction): the
         * difference of two such floats is hi - lo exactly, and subtracting
         * 2^23 gives lo exactly, so every lerp sees the values above */
        auto bt = [](uint32_t q, uint32_t k) {
            return __uint_as_float(__byte_perm(q, 0x4B000000u, 0x7440u + k));
        };
        const float2 mM = make_float2(-8388608.0f, -8388608.0f);
        /* quad bytes 0..3: c0..c3 of slice z (T.q[0]), c4..c7 of z + 1 */
        const float2 lo0 = make_float2(bt(T.q[0], 0), bt(T.q[1], 0));
        const float2 hi0 = make_float2(bt(T.q[0], 1), bt(T.q[1], 1));
        const float2 lo1 = make_float2(bt(T.q[0], 2), bt(T.q[1], 2));
        const float2 hi1 = make_float2(bt(T.q[0], 3), bt(T.q[1], 3));
        a02 = __ffma2_rn(__ffma2_rn(lo0, m1, hi0), fx, __fadd2_rn(lo0, mM));
        a13 = __ffma2_rn(__ffma2_rn(lo1, m1, hi1), fx, __fadd2_rn(lo1, mM));
    }
    else
    {
        const float2 lo0 = make_float2(T.c[0], T.c[4]), hi0 = make_float2(T.c[1], T.c[5]);
        const float2 lo1 = make_float2(T.c[2], T.c[6]), hi1 = make_float2(T.c[3], T.c[7]);
        a02 = __ffma2_rn(__ffma2_rn(lo0, m1, hi0), fx, lo0);
        a13 = __ffma2_rn(__ffma2_rn(lo1, m1, hi1), fx, lo1);
    }
    const float2 b01 = __ffma2_rn(__ffma2_rn(a02, m1, a13), make_float2(T.fy, T.fy), a02);
    return fmaf(b01.y - b01.x, T.fz, b01.x);
}

/* Linear, clamp-to-edge lookup of the transfer function at voxel value v
 * (texel coordinate v * tf_mul + tf_add = density * tfn - 1/2), stored as
 * interleaved (value_i, value_{i+1} - value_i) pairs (last difference 0).
 * Clamping the coordinate to [0, tfn - 1] before splitting it gives the
 * same texel pair and weight as clamping the texel index after. */
template <int TFS, class HV>
__device__ __forceinline__ float4 tf_lookup(const HV& H, float v)
{
    const float s = fminf(fmaxf(fmaf(v, H.tf_mul, H.tf_add), 0.0f), H.tf_last);
    /* floor(s) (s in [0, tf_last]) by adding 2^23 rounding down: its bits
     * carry the integer, no conversion instruction */
    const float y = __fadd_rd(s, 8388608.0f);
    const int i0 = int(__float_as_uint(y) - 0x4B000000u);
    const float f = s - (y - 8388608.0f);
    /* TFS: the table is in shared memory (generic loads); else read-only
     * global memory, the texel pair's 32 bytes (value, difference) in one
     * 256-bit load: the table is a device allocation, so every pair is
     * 32-byte aligned */
    const float4* e = H.tf + 2 * i0;
    float4 a, b;
    if (TFS)
    {
        a = e[0];
        b = e[1];
    }
    else
        asm("{\n\t.reg .u64 g;\n\tcvta.to.global.u64 g, %8;\n\t"
            "ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [g];\n\t}"
            : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z),
              "=f"(b.w)
            : "l"(e));
    /* value + difference * f per channel, two channels per FFMA2 */
    const float2 f2 = make_float2(f, f);
    const float2 rg = __ffma2_rn(make_float2(b.x, b.y), f2, make_float2(a.x, a.y));
    const float2 ba = __ffma2_rn(make_float2(b.z, b.w), f2, make_float2(a.z, a.w));
    return make_float4(rg.x, rg.y, ba.x, ba.y);
}

__device__ __forceinline__ float Md(const float* m, int r, int c)
{
    return m[c * 4 + r];
}

struct RayGeom
{
    float dir[3];
    float tg, tlo, thi;
    bool hit;
};

/* Pixel (px, py) of the rendered rect as an index into the frame. */
__device__ __forceinline__ uint64_t frame_index(const RayView& V, uint32_t px, uint32_t py)
{
    return uint64_t(py + V.y0) * V.FW + (px + V.x0);
}

/* Ray through the centre of pixel (px, py) of the rendered rect (frame pixel
 * (x0 + px, y0 + py)); FP32 IEEE ops in fixed order. A pixel outside the
 * view's conservative screen rectangle of the volume's box (V.cull) misses
 * the box: it returns no hit without the set-up arithmetic, as the full
 * computation would (about 85 % of a 1080p orbit frame's pixels). */
__device__ __forceinline__ RayGeom ray_setup(const RayView& V, uint32_t px,
                                             uint32_t py)
{
    RayGeom g;
    const uint32_t fx = px + V.x0, fy = py + V.y0;
    if (fx < V.cull[0] || fx >= V.cull[2] || fy < V.cull[1] || fy >= V.cull[3])
    {
        g.dir[0] = g.dir[1] = g.dir[2] = 0.0f;
        g.tg = g.tlo = g.thi = 0.0f;
        g.hit = false;
        return g;
    }
    const float nx =
        __fsub_rn(__fdiv_rn(__fmul_rn(__fadd_rn(__uint2float_rn(px + V.x0), 0.5f), 2.0f),
                            __uint2float_rn(V.FW)),
                  1.0f);
    const float ny =
        __fsub_rn(__fdiv_rn(__fmul_rn(__fadd_rn(__uint2float_rn(py + V.y0), 0.5f), 2.0f),
                            __uint2float_rn(V.FH)),
                  1.0f);
    float e[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        e[i] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(Md(V.inv_p, i, 0), nx),
                                             __fmul_rn(Md(V.inv_p, i, 1), ny)),
                                   __fmul_rn(Md(V.inv_p, i, 2), -1.0f)),
                         __fmul_rn(Md(V.inv_p, i, 3), 1.0f));
    const float ep[3] = {__fdiv_rn(e[0], e[3]), __fdiv_rn(e[1], e[3]),
                         __fdiv_rn(e[2], e[3])};
    float d[3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
    {
        const float pw =
            __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(Md(V.inv_mv, i, 0), ep[0]),
                                          __fmul_rn(Md(V.inv_mv, i, 1), ep[1])),
                                __fmul_rn(Md(V.inv_mv, i, 2), ep[2])),
                      Md(V.inv_mv, i, 3));
        d[i] = __fsub_rn(pw, V.eye[i]);
    }
    const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]),
                                                     __fmul_rn(d[1], d[1])),
                                           __fmul_rn(d[2], d[2])));
#pragma unroll
    for (int i = 0; i < 3; ++i)
        g.dir[i] = __fdiv_rn(d[i], len);
    const float lenE = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(ep[0], ep[0]),
                                                      __fmul_rn(ep[1], ep[1])),
                                            __fmul_rn(ep[2], ep[2])));
    const float nz = __fdiv_rn(ep[2], lenE);
    const float tnp = __fdiv_rn(-V.nearp, nz);
    float tmin[3], tmax[3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
    {
        const float di = g.dir[i] == 0.0f ? 1e-10f : g.dir[i];
        const float inv = __fdiv_rn(1.0f, di);
        const float tb = __fmul_rn(inv, __fsub_rn(V.gmin[i], V.eye[i]));
        const float tt = __fmul_rn(inv, __fsub_rn(V.gmax[i], V.eye[i]));
        tmin[i] = smin(tt, tb);
        tmax[i] = smax(tt, tb);
    }
    const float t0 = smax(smax(tmin[0], tmin[1]), smax(tmin[0], tmin[2]));
    const float t1 = smin(smin(tmax[0], tmax[1]), smin(tmax[0], tmax[2]));
    g.hit = t0 <= t1;
    g.tg = t0;
    float tlo = smax(t0, tnp);
    float thi = t1;
    for (uint32_t c = 0; c < V.n_clip; ++c)
    {
        const float* cp = V.clip[c];
        float rn = __fadd_rn(__fadd_rn(__fmul_rn(g.dir[0], cp[0]), __fmul_rn(g.dir[1], cp[1])),
                             __fmul_rn(g.dir[2], cp[2]));
        if (rn == 0.0f)
            rn = 1e-10f;
        const float ne = __fadd_rn(__fadd_rn(__fmul_rn(cp[0], V.eye[0]), __fmul_rn(cp[1], V.eye[1])),
                                   __fmul_rn(cp[2], V.eye[2]));
        const float t = __fdiv_rn(-__fadd_rn(ne, cp[3]), rn);
        if (rn > 0.0f)
            tlo = smax(tlo, t);
        else
            thi = smin(thi, t);
    }
    g.tlo = tlo;
    g.thi = thi;
    return g;
}

/* State of one ray between two samples, so that a lane can take a number of
 * samples, stop, and go on later (the refill kernels below). */
struct RayState
{
    float dir[3];
    float tg, thi;
    float kf;            /* index of the next sample (exact in FP32 below 2^24) */
    float kf_safe;       /* samples up to this index stay in the current brick */
    uint32_t err;        /* FC_ERROR value to report when the ray ends (0: none) */
    float4 dst;
    uint32_t entry;      /* leaf entry of the current brick (or empty cell) */
    const uint8_t* brick;
    /* slot coordinate of a sample of the brick: sc = fma(t, sa, sb), the
     * composition of the position, cell and slot maps (a few ulp from the
     * oracle's three-FMA chain; which brick a sample reads is exact) */
    float sa[3], sb[3];
};

/* First sample on the global grid at or after tlo; false: no sample. */
__device__ __forceinline__ bool ray_begin(const RayGeom& g, float step, RayState& r)
{
    r.dst = make_float4(0.f, 0.f, 0.f, 0.f);
    if (!g.hit || !(g.tlo <= g.thi))
        return false;
    int k = 0;
    if (g.tlo > g.tg)
        k = int(ceilf(__fdiv_rn(__fsub_rn(g.tlo, g.tg), step)));
    r.kf = __int2float_rn(k);
#pragma unroll
    for (int a = 0; a < 3; ++a)
    {
        r.dir[a] = g.dir[a];
        r.sa[a] = 0.f;
        r.sb[a] = 0.f;
    }
    r.tg = g.tg;
    r.thi = g.thi;
    r.kf_safe = -1.0f;
    r.err = 0u;
    r.entry = kLeafEmpty;
    r.brick = nullptr;
    return true;
}

/* Sample position in leaf-cell units at ray parameter t: single-rounding
 * FMAs in a fixed order (the CPU oracle evaluates the same fmaf chain). */
__device__ __forceinline__ void sample_cell_coord(const RayView& V, const RayState& r, float t,
                                                  float f[3])
{
#pragma unroll
    for (int a = 0; a < 3; ++a)
        f[a] = fmaf(fmaf(r.dir[a], t, V.eye[a]), V.gscale[a], V.goff[a]);
}

/* Leaf cell of a sample at cell coordinate f on one axis, or dims (outside
 * the octree). The sample's parameter is in [tnearGlobal, tfarGlobal), so it
 * lies in the volume's box: a cell index rounded one past the box's face (a
 * sample on the entry or exit face, which the reference shader takes at
 * tnear = tnearGlobal, fragRayCast.glsl:142-147) is the face cell. The low
 * face is the box's on every axis (f = 0); the high face only on axes with
 * the most cells (bm): shorter axes end inside the box, as the node boxes
 * of LODNode.cpp:30-64 (cell side worldSize / maxBricks) do. */
__device__ __forceinline__ uint32_t face_cell(float f, uint32_t dims, uint32_t bm)
{
    const uint32_t c = uint32_t(max(__float2int_rd(f), 0));
    return dims == bm ? min(c, dims - 1u) : c;
}

/* The slow path of a sample (index r.kf, position f) that leaves the range
 * known to lie in the current brick: finds its leaf cell (face_cell), the
 * brick there, and how far the ray stays in that brick. False: the sample
 * is outside the octree.
 *
 * The cell of a sample is monotone in its index along each axis (t, the
 * position and f are monotone single-rounding functions of it, and floor is
 * monotone), so if the sample at index k lies in the brick's cube of leaf
 * cells, so does every sample between this one and k. k is the estimated
 * last sample before the exit (or the one before it), checked with the
 * exact per-sample arithmetic; samples up to r.kf_safe then skip the lookup
 * and take the same brick the per-sample lookup would. */
template <int FILTER>
__device__ __forceinline__ bool locate(const RayView& V, RayState& r, float step, const float f[3])
{
    const uint32_t bm = max(max(V.dims[0], V.dims[1]), V.dims[2]);
    uint32_t c[3];
    bool inside = true;
#pragma unroll
    for (int a = 0; a < 3; ++a)
    {
        c[a] = face_cell(f[a], V.dims[a], bm);
        inside = inside && c[a] < V.dims[a];
    }
    r.kf_safe = r.kf; /* this sample only, unless shown otherwise below */
    if (!inside)
        return false;
    uint32_t entry = __ldg(V.leaf + (c[2] * V.dims[1] + c[1]) * V.dims[0] + c[0]);
    if (entry != kLeafEmpty && ((entry & kLeafSlotMask) + V.brick_units > V.pool_units ||
                                (entry >> kLeafSlotBits) > V.Lf))
    {
        /* entry outside the pool: reported when the ray ends, so that the
         * sample loop stores nothing to memory */
        r.err = 3u;
        entry = kLeafEmpty;
    }
    r.entry = entry;
    /* an empty cell spans one leaf cell; a brick at level L spans 2^(Lf-L) */
    const uint32_t sh = entry == kLeafEmpty ? 0u : V.Lf - (entry >> kLeafSlotBits);
#pragma unroll
    for (int a = 0; a < 3; ++a)
        c[a] >>= sh; /* the brick's cube, in its own cells */
    if (entry != kLeafEmpty)
    {
        const float half_texel = FILTER == LV_FILTER_TRILINEAR ? 0.5f : 0.0f;
        r.brick = V.pool + uint64_t(entry & kLeafSlotMask) * kSlotUnit;
        const float inv_side = __int_as_float(int(127u - sh) << 23); /* 2^-sh */
#pragma unroll
        for (int a = 0; a < 3; ++a)
        {
            /* slot coordinate = f * vs + off (vs, off exact); composed with
             * f = (eye + dir * t) * gscale + goff into one map of t */
            const float vs = __uint2float_rn(V.B[a]) * inv_side;
            const float off =
                (__uint2float_rn(V.O[a]) - __uint2float_rn(c[a] * V.B[a])) - half_texel;
            r.sa[a] = r.dir[a] * V.gscale[a] * vs;
            r.sb[a] = fmaf(fmaf(V.eye[a], V.gscale[a], V.goff[a]), vs, off);
        }
    }
    /* estimated parameter where the ray leaves the cube */
    float tx = 3.0e38f;
#pragma unroll
    for (int a = 0; a < 3; ++a)
    {
        const float d = r.dir[a];
        if (d != 0.0f)
        {
            const uint32_t bound = d > 0.0f ? min((c[a] + 1u) << sh, V.dims[a]) : c[a] << sh;
            tx = fminf(tx, __fdividef(__fdividef(__uint2float_rn(bound) - V.goff[a],
                                                 V.gscale[a]) -
                                          V.eye[a],
                                      d));
        }
    }
    float ke = fminf(floorf(__fdividef(tx - r.tg, step)), 16777215.0f);
#pragma unroll 1
    for (int attempt = 0; attempt < 2 && ke > r.kf; ++attempt, ke -= 1.0f)
    {
        float g[3];
        sample_cell_coord(V, r, fmaf(ke, step, r.tg), g);
        bool in = true;
#pragma unroll
        for (int a = 0; a < 3; ++a)
        {
            const uint32_t ca = face_cell(g[a], V.dims[a], bm);
            in = in && ca < V.dims[a] && (ca >> sh) == c[a];
        }
        if (in)
        {
            r.kf_safe = ke;
            break;
        }
    }
    return true;
}

/* Advances the ray to its next sample (index r.kf) with one divergent
 * region, the brick lookup where the ray leaves its safe range; false once
 * the ray has left its segment. The sample's voxels are read into T only
 * when it has data (`valid`: inside the segment and in a rendered brick, not
 * outside the octree or in a cell no brick covers), by predicated loads, so
 * a sample without data costs no branch. */
template <int DT, int FILTER, int EDGE, class HV>
__device__ __forceinline__ bool fetch_sample(const RayView& V, const HV& H, RayState& r, float step,
                                         Taps<FILTER>& T, bool& valid)
{
    const float t = fmaf(r.kf, step, r.tg);
    const bool live = t < r.thi;
    if (live && !(r.kf <= r.kf_safe))
    {
        float f[3];
        sample_cell_coord(V, r, t, f);
        if (!locate<FILTER>(V, r, step, f))
            r.entry = kLeafEmpty; /* outside the octree: this sample has no data */
    }
    r.kf += 1.0f;
    valid = live && r.entry != kLeafEmpty;
    float sc[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
        sc[a] = fmaf(t, r.sa[a], r.sb[a]);
    load_taps<DT, FILTER, EDGE>(V, H, r.brick, sc, T, valid);
    return live;
}

/* Transfer function, opacity correction and front-to-back blending of one
 * sample (fragRayCast.glsl:103-111); false once the early-termination
 * opacity is reached. A sample without data (!valid) is blended with opacity
 * 0 (the colour and opacity stay bit for bit as they were) and not counted,
 * so the march needs no branch around it. */
template <int FILTER, int TFS, bool RAW, class HV>
__device__ __forceinline__ bool composite_sample(const HV& H, RayState& r, float ac,
                                                 const Taps<FILTER>& T, bool valid,
                                                 uint32_t& nsamp)
{
    const float4 src = tf_lookup<TFS>(H, interp<FILTER, RAW>(T));
    const float am = fminf(src.w, 1.0f - 1.0f / 256.0f);
    const float alpha = valid ? 1.0f - ex2_approx(ac * lg2_approx(1.0f - am)) : 0.0f;
    const float w = alpha * (1.0f - r.dst.w);
    r.dst.x = fmaf(src.x, w, r.dst.x);
    r.dst.y = fmaf(src.y, w, r.dst.y);
    r.dst.z = fmaf(src.z, w, r.dst.z);
    r.dst.w = fmaf(alpha, 1.0f - r.dst.w, r.dst.w);
    nsamp += valid ? 1u : 0u;
    return !(r.dst.w > H.early);
}

/* One sample of the ray, fetched and composited with one tap set: false
 * once the ray has ended or reached the early-termination opacity. */
template <int DT, int FILTER, int TFS, int EDGE, class HV>
__device__ __forceinline__ bool ray_step(const RayView& V, const HV& H, RayState& r, float step,
                                         float ac, uint32_t& nsamp)
{
    Taps<FILTER> T;
    bool valid;
    const bool live = fetch_sample<DT, FILTER, EDGE>(V, H, r, step, T, valid);
    const bool cont =
        composite_sample<FILTER, TFS, raw_taps<DT, FILTER, EDGE>()>(H, r, ac, T, valid, nsamp);
    return live && cont;
}

/* A ray has ended: report an index check it failed. */
__device__ __forceinline__ void flush_error(const RayView& V, const RayState& r)
{
    if (r.err)
        atomicExch(&V.counters[FC_ERROR], r.err);
}

/* Colour a ray starts from: the frame so far in a later pass of a
 * multi-pass frame (RenderPipeline.cpp:92-158 composites every pass into
 * the same render texture), else transparent black. */
__device__ __forceinline__ float4 initial_dst(const RayView& V, uint32_t px, uint32_t py)
{
    return V.accumulate ? V.out[frame_index(V, px, py)] : make_float4(0.f, 0.f, 0.f, 0.f);
}

/* The whole ray. LOOKAHEAD = 1 loads the voxels of sample k + 1 before
 * sample k is composited, so the two latency chains overlap (a lone long
 * ray runs faster; more registers per thread). Samples, values and the
 * compositing order are those of ray_step either way; after an early
 * termination the loads of one extra sample are dropped. */
template <int DT, int FILTER, int TFS, int EDGE, int LOOKAHEAD, class HV>
__device__ float4 march(const RayView& V, const HV& H, const RayGeom& g, float step,
                        float ac, uint32_t& nsamp,
                        float4 init = make_float4(0.f, 0.f, 0.f, 0.f))
{
    RayState r;
    if (!ray_begin(g, step, r) || init.w > H.early)
        return init;
    r.dst = init;
    if (!LOOKAHEAD)
    {
        while (ray_step<DT, FILTER, TFS, EDGE>(V, H, r, step, ac, nsamp))
        {
        }
        flush_error(V, r);
        return r.dst;
    }
    /* two tap sets in turn (no copy of the taps between samples): fetch the
     * next sample into one while the other is composited. A sample without
     * data is fetched and composited masked, so each sample has one
     * divergent region (a brick lookup) and one loop exit. */
    constexpr bool RAW = raw_taps<DT, FILTER, EDGE>();
    Taps<FILTER> T0, T1;
    bool v0, v1;
    bool live0 = fetch_sample<DT, FILTER, EDGE>(V, H, r, step, T0, v0);
    while (live0)
    {
        const bool live1 = fetch_sample<DT, FILTER, EDGE>(V, H, r, step, T1, v1);
        if (!(composite_sample<FILTER, TFS, RAW>(H, r, ac, T0, v0, nsamp) && live1))
            break;
        live0 = fetch_sample<DT, FILTER, EDGE>(V, H, r, step, T0, v0);
        if (!composite_sample<FILTER, TFS, RAW>(H, r, ac, T1, v1, nsamp))
            break;
    }
    flush_error(V, r);
    return r.dst;
}

/* The ray cast of a view whose frame will be rendered again
 * (RayView::skip_if_missing): every block of the launch returns at once. */
__device__ __forceinline__ bool skip_frame(const RayView& V)
{
    return V.skip_if_missing &&
           *static_cast<const volatile uint32_t*>(V.counters + FC_MISSING) != 0u;
}

/* LA: one-sample look-ahead */
template <int DT, int FILTER, int EDGE, int LA>
__global__ void __launch_bounds__(256) raycast_kernel(const RayView V)
{
    if (skip_frame(V))
        return;
    const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t py = blockIdx.y * blockDim.y + threadIdx.y;
    const uint32_t n = frame_samples(V);
    const float step = __fdiv_rn(1.0f, __uint2float_rn(n));
    const float ac = __fdiv_rn(32.0f, __uint2float_rn(n));
    uint32_t nsamp = 0;
    if (px < V.W && py < V.H)
    {
        const RayGeom g = ray_setup(V, px, py);
        const float4 r =
            march<DT, FILTER, 0, EDGE, LA>(V, V, g, step, ac, nsamp, initial_dst(V, px, py));
        V.out[frame_index(V, px, py)] = r;
    }
    /* warp-aggregated 64-bit sample count */
    unsigned long long s = nsamp;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        s += __shfl_down_sync(0xFFFFFFFFu, s, o);
    if ((threadIdx.x + threadIdx.y * blockDim.x) % 32 == 0 && s)
        atomicAdd(reinterpret_cast<unsigned long long*>(V.counters + FC_SAMPLES_LO), s);
}

/* Batched mode: one persistent launch renders the tiles of many views. Each
 * CTA pops (view, tile) work items from a device queue (one atomic per
 * tile), keeps the current view's constants (and optionally its transfer
 * function) in shared memory, and ray casts tile_w x tile_h pixels. */
template <int DT, int FILTER, int TF_SHARED, int EDGE>
__global__ void __launch_bounds__(256)
    raycast_persistent_kernel(const RayView* __restrict__ views, TileQueue Q)
{
    __shared__ RayView sV;
    __shared__ uint32_t s_item, s_view;
    extern __shared__ float4 s_tf[];
    const uint32_t n_views = *Q.n_views;
    const uint32_t total = Q.tile_start[n_views];
    if (threadIdx.x == 0)
        atomicCAS(Q.clock, 0ull, globaltimer());
    uint32_t cached = 0xFFFFFFFFu;
    float step = 0.f, ac = 0.f;
    HotView H{};
    for (;;)
    {
        if (threadIdx.x == 0)
        {
            uint32_t item = atomicAdd(Q.head, 1u);
            if (Q.order && item < total)
                item = Q.order[item];
            uint32_t lo = 0, hi = n_views;
            if (item < total)
                while (hi - lo > 1)
                {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (Q.tile_start[mid] <= item)
                        lo = mid;
                    else
                        hi = mid;
                }
            s_item = item;
            s_view = lo;
        }
        __syncthreads();
        const uint32_t item = s_item;
        const uint32_t gv = s_view;
        if (item >= total)
            break;
        const uint32_t v = Q.view_ids[gv];
        if (v != cached)
        {
            const uint32_t* src = reinterpret_cast<const uint32_t*>(views + v);
            uint32_t* dst = reinterpret_cast<uint32_t*>(&sV);
            for (uint32_t w = threadIdx.x; w < sizeof(RayView) / 4; w += blockDim.x)
                dst[w] = src[w];
            __syncthreads();
            if (TF_SHARED)
            {
                for (uint32_t i = threadIdx.x; i < 2u * sV.tfn; i += blockDim.x)
                    s_tf[i] = sV.tf[i];
                __syncthreads();
                if (threadIdx.x == 0)
                    sV.tf = s_tf;
                __syncthreads();
            }
            cached = v;
            H = hot_view(sV);
            const uint32_t n = sV.counters[FC_SAMPLES_PER_RAY];
            step = __fdiv_rn(1.0f, __uint2float_rn(n));
            ac = __fdiv_rn(32.0f, __uint2float_rn(n));
        }
        const uint32_t t = item - Q.tile_start[gv];
        const uint32_t tiles_x = (sV.W + Q.tile_w - 1) / Q.tile_w;
        const uint32_t px = (t % tiles_x) * Q.tile_w + threadIdx.x % Q.tile_w;
        const uint32_t py = (t / tiles_x) * Q.tile_h + threadIdx.x / Q.tile_w;
        uint32_t nsamp = 0;
        if (px < sV.W && py < sV.H && threadIdx.x < Q.tile_w * Q.tile_h)
        {
            const RayGeom g = ray_setup(sV, px, py);
            const float4 r = march<DT, FILTER, TF_SHARED, EDGE, 0>(sV, H, g, step, ac, nsamp);
            sV.out[frame_index(sV, px, py)] = r;
        }
        unsigned long long sum = nsamp;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            sum += __shfl_down_sync(0xFFFFFFFFu, sum, o);
        if ((threadIdx.x & 31u) == 0 && sum)
            atomicAdd(reinterpret_cast<unsigned long long*>(sV.counters + FC_SAMPLES_LO), sum);
        __syncthreads();
    }
    if (threadIdx.x == 0)
        atomicMax(Q.clock + 1, globaltimer());
}

/* Longest-first tile order of one view. A tile's cost is estimated by the
 * length of its centre ray inside the volume (near and clip planes
 * applied), quantised to kTileBuckets classes; a counting sort lists the
 * longest class first (the order within a class does not matter: every
 * pixel is computed independently). hist[0, kTileBuckets) are the class
 * counts and hist[kTileBuckets, 2 kTileBuckets) the scatter cursors, both
 * zeroed before the key pass. */
constexpr uint32_t kTileBuckets = 64;

/* Slot of an item of class `key` in the sorted order: the class's first
 * slot (base, shared memory) plus the item's rank among the class's items
 * claimed so far, one global atomic per class present in the warp (items of
 * one class are many: per-item atomics on one cursor serialised). key =
 * kTileBuckets: no item (the lane still takes part in the warp-wide
 * match). */
__device__ __forceinline__ uint32_t base_of_item(const uint32_t* base, uint32_t* hist,
                                                 uint32_t key)
{
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t leader = __ffs(peers) - 1u;
    uint32_t first = 0;
    if (lane == leader && key < kTileBuckets)
        first = atomicAdd(&hist[kTileBuckets + key], __popc(peers));
    first = __shfl_sync(0xFFFFFFFFu, first, leader); /* each lane: its class's leader */
    const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
    return key < kTileBuckets ? base[key] + first + rank : 0xFFFFFFFFu;
}

__global__ void __launch_bounds__(256)
    tile_key_kernel(const RayView V, uint32_t tile_w, uint32_t tile_h, uint32_t tiles_x,
                    uint32_t total, float buckets_per_length, uint8_t* __restrict__ keys,
                    uint32_t* __restrict__ hist)
{
    __shared__ uint32_t h[kTileBuckets];
    for (uint32_t i = threadIdx.x; i < kTileBuckets; i += blockDim.x)
        h[i] = 0;
    __syncthreads();
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < total)
    {
        const uint32_t px = min((t % tiles_x) * tile_w + tile_w / 2, V.W - 1);
        const uint32_t py = min((t / tiles_x) * tile_h + tile_h / 2, V.H - 1);
        const RayGeom g = ray_setup(V, px, py);
        const float len = g.hit && g.tlo <= g.thi ? g.thi - g.tlo : 0.0f;
        const uint32_t q = uint32_t(fminf(len * buckets_per_length, float(kTileBuckets - 1)));
        const uint32_t key = kTileBuckets - 1u - q;
        keys[t] = uint8_t(key);
        atomicAdd(&h[key], 1u);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < kTileBuckets; i += blockDim.x)
        if (h[i])
            atomicAdd(&hist[i], h[i]);
}

__global__ void __launch_bounds__(256)
    tile_order_kernel(const uint8_t* __restrict__ keys, uint32_t* __restrict__ hist,
                      uint32_t* __restrict__ order, uint32_t total)
{
    __shared__ uint32_t base[kTileBuckets];
    /* class counts loaded in parallel, then one thread scans them in shared
     * memory (a serial scan over global memory cost ~14 us per launch) */
    if (threadIdx.x < kTileBuckets)
        base[threadIdx.x] = hist[threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 0)
    {
        uint32_t acc = 0;
        for (uint32_t k = 0; k < kTileBuckets; ++k)
        {
            const uint32_t c = base[k];
            base[k] = acc;
            acc += c;
        }
    }
    __syncthreads();
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t key = t < total ? keys[t] : kTileBuckets;
    const uint32_t pos = base_of_item(base, hist, key);
    if (t < total && pos < total)
        order[pos] = t;
}

/* Single view on a resident grid: CTAs take tile_w x tile_h pixel tiles
 * (one ray per thread) from a device queue, the view's FC_QUEUE counter. */
template <int DT, int FILTER, int EDGE, int LA>
__global__ void __launch_bounds__(256)
    raycast_queue_kernel(const RayView V, uint32_t tile_w, uint32_t tile_h,
                         const uint32_t* __restrict__ order)
{
    if (skip_frame(V))
        return;
    __shared__ uint32_t s_item;
    const uint32_t n = frame_samples(V);
    const float step = __fdiv_rn(1.0f, __uint2float_rn(n));
    const float ac = __fdiv_rn(32.0f, __uint2float_rn(n));
    const uint32_t tiles_x = (V.W + tile_w - 1) / tile_w;
    const uint32_t total = tiles_x * ((V.H + tile_h - 1) / tile_h);
    const uint32_t tx = threadIdx.x % tile_w, ty = threadIdx.x / tile_w;
    uint32_t nsamp = 0;
    for (;;)
    {
        if (threadIdx.x == 0)
            s_item = atomicAdd(V.counters + FC_QUEUE, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        __syncthreads();
        if (item >= total)
            break;
        const uint32_t tile = order ? order[item] : item;
        const uint32_t px = (tile % tiles_x) * tile_w + tx;
        const uint32_t py = (tile / tiles_x) * tile_h + ty;
        if (px < V.W && py < V.H)
        {
            const RayGeom g = ray_setup(V, px, py);
            V.out[frame_index(V, px, py)] =
                march<DT, FILTER, 0, EDGE, LA>(V, V, g, step, ac, nsamp, initial_dst(V, px, py));
        }
    }
    unsigned long long sum = nsamp;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        sum += __shfl_down_sync(0xFFFFFFFFu, sum, o);
    if ((threadIdx.x & 31u) == 0 && sum)
        atomicAdd(reinterpret_cast<unsigned long long*>(V.counters + FC_SAMPLES_LO), sum);
}

/* One CTA per tile: block i renders tile order[i] (or tile i). */
template <int DT, int FILTER, int EDGE, int LA>
__global__ void __launch_bounds__(256)
    raycast_tiles_kernel(const RayView V, uint32_t tile_w, uint32_t tile_h,
                         const uint32_t* __restrict__ order)
{
    if (skip_frame(V))
        return;
    const uint32_t n = frame_samples(V);
    const float step = __fdiv_rn(1.0f, __uint2float_rn(n));
    const float ac = __fdiv_rn(32.0f, __uint2float_rn(n));
    const uint32_t tiles_x = (V.W + tile_w - 1) / tile_w;
    const uint32_t tile = order ? order[blockIdx.x] : blockIdx.x;
    const uint32_t px = (tile % tiles_x) * tile_w + threadIdx.x % tile_w;
    const uint32_t py = (tile / tiles_x) * tile_h + threadIdx.x / tile_w;
    uint32_t nsamp = 0;
    if (px < V.W && py < V.H)
    {
        const RayGeom g = ray_setup(V, px, py);
        V.out[frame_index(V, px, py)] =
            march<DT, FILTER, 0, EDGE, LA>(V, V, g, step, ac, nsamp, initial_dst(V, px, py));
    }
    unsigned long long sum = nsamp;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        sum += __shfl_down_sync(0xFFFFFFFFu, sum, o);
    if ((threadIdx.x & 31u) == 0 && sum)
        atomicAdd(reinterpret_cast<unsigned long long*>(V.counters + FC_SAMPLES_LO), sum);
}

/* Resident grid, warp-granular queue: each warp pops a 32-pixel tile (one
 * ray per lane) from the view's FC_QUEUE counter, in the given order. */
template <int DT, int FILTER, int EDGE, int LA>
__global__ void __launch_bounds__(128)
    raycast_warp_tiles_kernel(const RayView V, uint32_t tile_w, uint32_t tile_h,
                              const uint32_t* __restrict__ order)
{
    if (skip_frame(V))
        return;
    const uint32_t n = frame_samples(V);
    const float step = __fdiv_rn(1.0f, __uint2float_rn(n));
    const float ac = __fdiv_rn(32.0f, __uint2float_rn(n));
    const uint32_t tiles_x = (V.W + tile_w - 1) / tile_w;
    const uint32_t total = tiles_x * ((V.H + tile_h - 1) / tile_h);
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t nsamp = 0;
    for (;;)
    {
        uint32_t item = 0;
        if (lane == 0)
            item = atomicAdd(V.counters + FC_QUEUE, 1u);
        item = __shfl_sync(0xFFFFFFFFu, item, 0);
        if (item >= total)
            break;
        const uint32_t tile = order ? order[item] : item;
        const uint32_t px = (tile % tiles_x) * tile_w + lane % tile_w;
        const uint32_t py = (tile / tiles_x) * tile_h + lane / tile_w;
        if (px < V.W && py < V.H)
        {
            const RayGeom g = ray_setup(V, px, py);
            V.out[frame_index(V, px, py)] =
                march<DT, FILTER, 0, EDGE, LA>(V, V, g, step, ac, nsamp, initial_dst(V, px, py));
        }
        __syncwarp();
    }
    unsigned long long sum = nsamp;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        sum += __shfl_down_sync(0xFFFFFFFFu, sum, o);
    if (lane == 0 && sum)
        atomicAdd(reinterpret_cast<unsigned long long*>(V.counters + FC_SAMPLES_LO), sum);
}

/* ---------------------------------------------------------------- refill
 * Persistent ray cast with lane refill. Every warp takes tile_w x tile_h
 * pixel tiles from a device queue (one atomic per tile) and hands the tile's
 * pixels to its lanes in order; a lane whose ray has finished takes the next
 * pixel at the next check (every `checks` samples), so lanes do not idle
 * while the longest ray of their warp finishes. When a tile runs out, the
 * warp takes the next one of the same view without waiting for its lanes;
 * a tile of another view (batched launch) is started once the warp has
 * drained. Each ray takes exactly the samples of march() in the same
 * order, so the image is identical to the one-thread-per-pixel kernel's. */
constexpr uint32_t kRefillThreads = 128;
constexpr uint32_t kRefillMinCtas = 8; /* 32 warps per SM: at most 64 registers */
constexpr uint32_t kFull = 0xFFFFFFFFu;
constexpr uint32_t kNoItem = 0xFFFFFFFFu;

__device__ __forceinline__ uint32_t warp_pop(uint32_t* head)
{
    uint32_t v = 0;
    if ((threadIdx.x & 31u) == 0)
        v = atomicAdd(head, 1u);
    return __shfl_sync(kFull, v, 0);
}

/* group view of a work item: tile_start is ascending, tile_start[0] = 0 */
__device__ __forceinline__ uint32_t find_view(const TileQueue& Q, uint32_t n_views,
                                              uint32_t item)
{
    uint32_t lo = 0, hi = n_views;
    while (hi - lo > 1)
    {
        const uint32_t mid = (lo + hi) >> 1;
        if (Q.tile_start[mid] <= item)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

__device__ __forceinline__ void load_view(RayView* dst, const RayView* src)
{
    __syncwarp();
    const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
    uint32_t* d = reinterpret_cast<uint32_t*>(dst);
    for (uint32_t w = threadIdx.x & 31u; w < sizeof(RayView) / 4; w += 32)
        d[w] = s[w];
    __syncwarp();
}

/* Longest-first order of the work items of one batched group. The cost of
 * a (view, tile) item is estimated as the samples of the tile's centre ray,
 * its length inside the volume times the view's samples per unit length,
 * in classes of a quarter octave; a counting sort lists the costliest
 * class first. hist holds the class counts then the scatter cursors, both
 * zeroed before the key pass. */
__global__ void __launch_bounds__(256)
    batch_key_kernel(const RayView* __restrict__ views, TileQueue Q, uint8_t* __restrict__ keys,
                     uint32_t* __restrict__ hist)
{
    __shared__ uint32_t h[kTileBuckets];
    for (uint32_t i = threadIdx.x; i < kTileBuckets; i += blockDim.x)
        h[i] = 0;
    __syncthreads();
    const uint32_t n_views = *Q.n_views;
    const uint32_t total = Q.tile_start[n_views];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += gridDim.x * blockDim.x)
    {
        const uint32_t gv = find_view(Q, n_views, i);
        const RayView& V = views[Q.view_ids[gv]];
        const uint32_t tile = i - Q.tile_start[gv];
        const uint32_t tiles_x = (V.W + Q.tile_w - 1) / Q.tile_w;
        const uint32_t px = min((tile % tiles_x) * Q.tile_w + Q.tile_w / 2, V.W - 1);
        const uint32_t py = min((tile / tiles_x) * Q.tile_h + Q.tile_h / 2, V.H - 1);
        const RayGeom g = ray_setup(V, px, py);
        const float len = g.hit && g.tlo <= g.thi ? g.thi - g.tlo : 0.0f;
        const float est = len * __uint2float_rn(V.counters[FC_SAMPLES_PER_RAY]);
        const uint32_t q = uint32_t(fminf(log2f(est + 1.0f) * 4.0f, float(kTileBuckets - 1)));
        const uint32_t key = kTileBuckets - 1u - q;
        keys[i] = uint8_t(key);
        atomicAdd(&h[key], 1u);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < kTileBuckets; i += blockDim.x)
        if (h[i])
            atomicAdd(&hist[i], h[i]);
}

__global__ void __launch_bounds__(256)
    batch_order_kernel(TileQueue Q, const uint8_t* __restrict__ keys,
                       uint32_t* __restrict__ hist, uint32_t* __restrict__ order)
{
    __shared__ uint32_t base[kTileBuckets];
    /* class counts loaded in parallel, then one thread scans them in shared
     * memory (a serial scan over global memory cost ~14 us per launch) */
    if (threadIdx.x < kTileBuckets)
        base[threadIdx.x] = hist[threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 0)
    {
        uint32_t acc = 0;
        for (uint32_t k = 0; k < kTileBuckets; ++k)
        {
            const uint32_t c = base[k];
            base[k] = acc;
            acc += c;
        }
    }
    __syncthreads();
    const uint32_t total = Q.tile_start[*Q.n_views];
    /* warp-uniform trip count: every lane reaches the warp-wide match */
    for (uint32_t b0 = blockIdx.x * blockDim.x; b0 < total; b0 += gridDim.x * blockDim.x)
    {
        const uint32_t i = b0 + threadIdx.x;
        const uint32_t key = i < total ? keys[i] : kTileBuckets;
        const uint32_t pos = base_of_item(base, hist, key);
        if (i < total && pos < total)
            order[pos] = i;
    }
}

__device__ __forceinline__ void flush_samples(const RayView& V, uint32_t nsamp)
{
    unsigned long long s = nsamp;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        s += __shfl_down_sync(kFull, s, o);
    if ((threadIdx.x & 31u) == 0 && s)
        atomicAdd(reinterpret_cast<unsigned long long*>(V.counters + FC_SAMPLES_LO), s);
}

struct ViewConsts
{
    float step, ac;
    uint32_t tiles_x;
};

__device__ __forceinline__ ViewConsts view_consts(const RayView& V, uint32_t tile_w)
{
    ViewConsts k;
    const uint32_t n = view_samples(V);
    k.step = __fdiv_rn(1.0f, __uint2float_rn(n));
    k.ac = __fdiv_rn(32.0f, __uint2float_rn(n));
    k.tiles_x = (V.W + tile_w - 1) / tile_w;
    return k;
}

/* MULTI: V is this warp's shared copy `sv` of the current view, reloaded
 * from `views` on a view change; else V is the launch's single view. */
template <int DT, int FILTER, int EDGE, bool MULTI>
__device__ __forceinline__ void refill_body(const RayView& V, RayView* sv,
                                            const RayView* __restrict__ views,
                                            const TileQueue& Q, uint32_t* head,
                                            uint32_t n_views, uint32_t total, uint32_t checks,
                                            const uint32_t* __restrict__ order)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t below = (1u << lane) - 1u;
    const uint32_t tw = Q.tile_w, th = Q.tile_h, npix = tw * th;
    uint32_t item = warp_pop(head);
    if (item >= total)
        return;
    uint32_t gv = 0;
    if (MULTI)
    {
        gv = find_view(Q, n_views, item);
        load_view(sv, views + Q.view_ids[gv]);
    }
    ViewConsts K = view_consts(V, tw);
    uint32_t tile = MULTI ? item - Q.tile_start[gv] : (order ? order[item] : item);
    uint32_t next = 0, pending = kNoItem;
    bool exhausted = false, active = false;
    uint32_t px = 0, py = 0, nsamp = 0;
    RayState r;
    for (;;)
    {
        /* hand the tile's next pixels to idle lanes, in lane order */
        for (;;)
        {
            const uint32_t idle = __ballot_sync(kFull, !active);
            if (!idle)
                break;
            if (next >= npix)
            {
                if (exhausted || pending != kNoItem)
                    break;
                const uint32_t nitem = warp_pop(head);
                if (nitem >= total)
                {
                    exhausted = true;
                    break;
                }
                if (MULTI && find_view(Q, n_views, nitem) != gv)
                {
                    pending = nitem; /* another view: drain first */
                    break;
                }
                tile = MULTI ? nitem - Q.tile_start[gv] : (order ? order[nitem] : nitem);
                next = 0;
            }
            const uint32_t mine = next + __popc(idle & below);
            next = min(next + uint32_t(__popc(idle)), npix);
            if (!active && mine < npix)
            {
                px = (tile % K.tiles_x) * tw + mine % tw;
                py = (tile / K.tiles_x) * th + mine / tw;
                if (px < V.W && py < V.H)
                {
                    const RayGeom g = ray_setup(V, px, py);
                    const float4 init = initial_dst(V, px, py);
                    active = ray_begin(g, K.step, r) && !(init.w > V.early);
                    r.dst = init;
                    if (!active)
                        V.out[frame_index(V, px, py)] = init;
                }
            }
        }
        if (!__any_sync(kFull, active))
        {
            if (MULTI && pending != kNoItem)
            {
                flush_samples(V, nsamp);
                nsamp = 0;
                gv = find_view(Q, n_views, pending);
                load_view(sv, views + Q.view_ids[gv]);
                K = view_consts(V, tw);
                tile = pending - Q.tile_start[gv];
                pending = kNoItem;
                next = 0;
                continue;
            }
            break; /* queue exhausted and every lane done */
        }
        if (active)
            for (uint32_t k = 0; k < checks; ++k)
                if (!ray_step<DT, FILTER, 0, EDGE>(V, V, r, K.step, K.ac, nsamp))
                {
                    active = false;
                    V.out[frame_index(V, px, py)] = r.dst;
                    flush_error(V, r);
                    break;
                }
    }
    flush_samples(V, nsamp);
}

/* Single view (lv_render): the queue head is the view's FC_QUEUE counter. */
template <int DT, int FILTER, int EDGE>
__global__ void __launch_bounds__(kRefillThreads, kRefillMinCtas)
    raycast_refill_kernel(const RayView V, uint32_t tile_w, uint32_t tile_h, uint32_t checks,
                          const uint32_t* __restrict__ order)
{
    if (skip_frame(V))
        return;
    TileQueue Q{};
    Q.tile_w = tile_w;
    Q.tile_h = tile_h;
    frame_samples(V);
    const uint32_t tiles = ((V.W + tile_w - 1) / tile_w) * ((V.H + tile_h - 1) / tile_h);
    refill_body<DT, FILTER, EDGE, false>(V, nullptr, nullptr, Q, V.counters + FC_QUEUE, 1u,
                                         tiles, checks, order);
}

/* Batched: tiles of many views of one kernel variant. */
template <int DT, int FILTER, int EDGE>
__global__ void __launch_bounds__(kRefillThreads, kRefillMinCtas)
    raycast_refill_views_kernel(const RayView* __restrict__ views, TileQueue Q, uint32_t checks)
{
    __shared__ RayView sV[kRefillThreads / 32];
    if (threadIdx.x == 0)
        atomicCAS(Q.clock, 0ull, globaltimer());
    const uint32_t n_views = *Q.n_views;
    RayView* sv = sV + (threadIdx.x >> 5);
    refill_body<DT, FILTER, EDGE, true>(*sv, sv, views, Q, Q.head, n_views,
                                        Q.tile_start[n_views], checks, nullptr);
    if ((threadIdx.x & 31u) == 0)
        atomicMax(Q.clock + 1, globaltimer());
}

__global__ void to_rgba8_kernel(const float4* __restrict__ in,
                                uchar4* __restrict__ out, uint64_t n)
{
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
         i += uint64_t(gridDim.x) * blockDim.x)
    {
        const float4 c = in[i];
        const auto q = [](float v) {
            return (unsigned char)(fminf(fmaxf(v, 0.0f), 1.0f) * 255.0f);
        };
        out[i] = make_uchar4(q(c.x), q(c.y), q(c.z), 255);
    }
}

} // namespace

lv_status launch_resolve(lv_ctx* ctx, const ResolveView& R, cudaStream_t s)
{
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    resolve_kernel<<<sms, 256, 0, s>>>(R);
    LV_CUDA(ctx, cudaGetLastError());
    return LV_OK;
}

lv_status launch_leaf_fill(lv_ctx* ctx, const ResolveView& R, cudaStream_t s)
{
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    if (!R.synchronous) /* ancestors may shadow entries: drop them */
        prune_kernel<<<sms, 256, 0, s>>>(R);
    LV_CUDA(ctx, cudaGetLastError());
    leaf_fill_kernel<<<2 * sms, 256, 0, s>>>(R);
    LV_CUDA(ctx, cudaGetLastError());
    return LV_OK;
}

namespace
{
/* CTAs of `kernel` resident on the whole GPU at once (occupancy API). */
template <typename K>
uint32_t resident_ctas(lv_ctx* ctx, K kernel, int threads, size_t smem)
{
    int per_sm = 0, sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) !=
            cudaSuccess ||
        per_sm < 1)
    {
        cudaGetLastError();
        per_sm = 1;
    }
    return uint32_t(per_sm) * uint32_t(sms);
}

/* One instantiation per (voxel type, filter, TF staging, edge clamping);
 * ctas = 0: as many CTAs as are resident at once. */
template <int DT, int F, int TFS, int EDGE>
lv_status persistent_dispatch(lv_ctx* ctx, const RayView* d_rays, const TileQueue& Q,
                              uint32_t ctas, size_t smem, cudaStream_t s)
{
    auto k = raycast_persistent_kernel<DT, F, TFS, EDGE>;
    if (smem > 48 * 1024)
        LV_CUDA(ctx, cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          int(smem)));
    const int threads = int(Q.tile_w * Q.tile_h);
    uint32_t grid = resident_ctas(ctx, k, threads, smem);
    if (ctas)
    {
        int sms = 152;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
        grid = uint32_t(sms) * ctas;
    }
    k<<<grid, threads, smem, s>>>(d_rays, Q);
    LV_CUDA(ctx, cudaGetLastError());
    return LV_OK;
}

template <int DT, int F, int EDGE>
lv_status refill_views_dispatch(lv_ctx* ctx, const RayView* d_rays, const TileQueue& Q,
                                uint32_t ctas, uint32_t checks, cudaStream_t s)
{
    auto k = raycast_refill_views_kernel<DT, F, EDGE>;
    uint32_t grid = resident_ctas(ctx, k, kRefillThreads, 0);
    if (ctas)
    {
        int sms = 152;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
        grid = uint32_t(sms) * ctas;
    }
    k<<<grid, kRefillThreads, 0, s>>>(d_rays, Q, checks);
    LV_CUDA(ctx, cudaGetLastError());
    return LV_OK;
}

/* A fixed-pitch kernel decides the brick layout from its pitch at compile
 * time (voxel quads for uint8 rows of kQuadMinRow to kQuadMaxRow); a view
 * whose pool keeps such bricks compact (LV_BRICKS_COMPACT) takes the
 * generic-pitch kernels, which read the layout from the view. */
bool fixed_pitch_layout(const RayView& V)
{
    return V.dtype != LV_DT_UINT8 || (V.quads != 0) == quad_layout(V.dtype, V.N[0]);
}

/* Scratch bytes of the longest-first order of V's tiles. */
size_t order_bytes_of(const RayView& V, const lv_render_launch& L)
{
    const size_t total =
        size_t((V.W + L.tile_w - 1) / L.tile_w) * ((V.H + L.tile_h - 1) / L.tile_h);
    return 2 * kTileBuckets * sizeof(uint32_t) + ((total + 15) & ~size_t(15)) +
           sizeof(uint32_t) * total;
}

/* Longest-first order of the tiles of V (a memset and two small launches)
 * in `scratch` (tile_order_bytes); nullptr for raster order. */
const uint32_t* tile_order(lv_ctx* ctx, const RayView& V, const lv_render_launch& L,
                           uint8_t* scratch, cudaStream_t s, lv_status& st)
{
    st = LV_OK;
    if (L.order != LV_ORDER_LONGEST_FIRST)
        return nullptr;
    const uint32_t tiles_x = (V.W + L.tile_w - 1) / L.tile_w;
    const uint32_t total = tiles_x * ((V.H + L.tile_h - 1) / L.tile_h);
    const size_t hist_bytes = 2 * kTileBuckets * sizeof(uint32_t);
    const size_t key_bytes = (size_t(total) + 15) & ~size_t(15);
    cudaError_t e = cudaMemsetAsync(scratch, 0, hist_bytes, s);
    if (e != cudaSuccess)
    {
        st = cuda_fail(ctx, e, "tile order");
        return nullptr;
    }
    uint32_t* hist = reinterpret_cast<uint32_t*>(scratch);
    uint8_t* keys = scratch + hist_bytes;
    uint32_t* order = reinterpret_cast<uint32_t*>(keys + key_bytes);
    float diag = 0.f;
    for (int a = 0; a < 3; ++a)
        diag += (V.gmax[a] - V.gmin[a]) * (V.gmax[a] - V.gmin[a]);
    const float per_length = float(kTileBuckets) / std::sqrt(diag);
    const uint32_t blocks = (total + 255) / 256;
    tile_key_kernel<<<blocks, 256, 0, s>>>(V, L.tile_w, L.tile_h, tiles_x, total, per_length,
                                           keys, hist);
    tile_order_kernel<<<blocks, 256, 0, s>>>(keys, hist, order, total);
    e = cudaGetLastError();
    if (e != cudaSuccess)
    {
        st = cuda_fail(ctx, e, "tile order");
        return nullptr;
    }
    return order;
}

/* lv_render's scratch for the tile order of V. */
uint8_t* render_order_scratch(lv_ctx* ctx, const RayView& V, const lv_render_launch& L,
                              lv_status& st)
{
    st = LV_OK;
    if (L.order != LV_ORDER_LONGEST_FIRST)
        return nullptr;
    DeviceBuffer& buf = ctx->renderer->tiles;
    const cudaError_t e = buf.reserve(order_bytes_of(V, L));
    if (e != cudaSuccess)
        st = cuda_fail(ctx, e, "tile order");
    return buf.as<uint8_t>();
}

} // namespace

lv_render_launch effective_launch(const RayView& V, const lv_render_launch& L)
{
    if (V.dtype == LV_DT_UINT8 || V.dtype == LV_DT_UINT16)
        return L;
    lv_render_launch T = L;
    T.kind = LV_LAUNCH_TILE_GRID;
    const uint32_t px = T.tile_w * T.tile_h;
    if (px == 0 || px > 256 || px % 32 != 0)
    {
        T.tile_w = 8;
        T.tile_h = 16;
    }
    return T;
}

lv_status prepare_frame_order(lv_ctx* ctx, const RayView& V, const lv_render_launch& L,
                              cudaStream_t side, const uint32_t*& order)
{
    order = nullptr;
    const lv_render_launch T = effective_launch(V, L);
    if (T.kind == LV_LAUNCH_GRID || T.order != LV_ORDER_LONGEST_FIRST)
        return LV_OK;
    lv_status st = LV_OK;
    uint8_t* scratch = render_order_scratch(ctx, V, T, st);
    if (st != LV_OK)
        return st;
    order = tile_order(ctx, V, T, scratch, side, st);
    return st;
}

namespace
{
/* The tile order of a launch: the one lv_render computed ahead for this
 * frame on its side stream (scratch == nullptr: lv_render's own scratch),
 * else computed now on `s` (null for raster order). */
const uint32_t* frame_order(lv_ctx* ctx, const RayView& V, const lv_render_launch& L,
                            uint8_t* scratch, cudaStream_t s, lv_status& st)
{
    st = LV_OK;
    if (!scratch && ctx->renderer->pre_order)
        return ctx->renderer->pre_order;
    if (!scratch)
        scratch = render_order_scratch(ctx, V, L, st);
    if (st != LV_OK)
        return nullptr;
    return tile_order(ctx, V, L, scratch, s, st);
}

template <int DT, int F, int EDGE>
lv_status refill_dispatch(lv_ctx* ctx, const RayView& V, const lv_render_launch& L,
                          cudaStream_t s)
{
    lv_status st = LV_OK;
    const uint32_t* order = frame_order(ctx, V, L, nullptr, s, st);
    if (st != LV_OK)
        return st;
    auto k = raycast_refill_kernel<DT, F, EDGE>;
    const uint32_t tiles = ((V.W + L.tile_w - 1) / L.tile_w) * ((V.H + L.tile_h - 1) / L.tile_h);
    const uint32_t warps = kRefillThreads / 32;
    const uint32_t grid = std::max(1u, std::min(resident_ctas(ctx, k, kRefillThreads, 0),
                                                (tiles + warps - 1) / warps));
    k<<<grid, kRefillThreads, 0, s>>>(V, L.tile_w, L.tile_h, L.samples_per_check, order);
    LV_CUDA(ctx, cudaGetLastError());
    return LV_OK;
}

/* One CTA per tile (LV_LAUNCH_TILE_GRID). */
template <int DT, int F, int EDGE, int LA>
lv_status tiles_dispatch(lv_ctx* ctx, const RayView& V, const lv_render_launch& L,
                         cudaStream_t s, uint8_t* scratch)
{
    lv_status st = LV_OK;
    const uint32_t* order = frame_order(ctx, V, L, scratch, s, st);
    if (st != LV_OK)
        return st;
    const uint32_t tiles = ((V.W + L.tile_w - 1) / L.tile_w) * ((V.H + L.tile_h - 1) / L.tile_h);
    raycast_tiles_kernel<DT, F, EDGE, LA><<<tiles, L.tile_w * L.tile_h, 0, s>>>(V, L.tile_w,
                                                                            L.tile_h, order);
    LV_CUDA(ctx, cudaGetLastError());
    return LV_OK;
}

/* The voxel types other than uint8 / uint16 (kDtAny kernels, the voxel type a
 * run-time switch) always use one CTA per tile, with the launch's tile shape
 * (8 x 16 when it is not a CTA's), order and look-ahead. */
template <int F, int EDGE>
lv_status any_type_dispatch(lv_ctx* ctx, const RayView& V, const lv_render_launch& L,
                            cudaStream_t s, uint8_t* scratch)
{
    const lv_render_launch T = effective_launch(V, L);
    return T.lookahead ? tiles_dispatch<kDtAny, F, EDGE, 1>(ctx, V, T, s, scratch)
                       : tiles_dispatch<kDtAny, F, EDGE, 0>(ctx, V, T, s, scratch);
}

template <int DT, int F, int EDGE, int LA>
lv_status plain_dispatch_la(lv_ctx* ctx, const RayView& V, const lv_render_launch& L,
                            cudaStream_t s, uint8_t* scratch)
{
    if (L.kind == LV_LAUNCH_WARP_TILES)
    {
        lv_status st = LV_OK;
        const uint32_t* order = frame_order(ctx, V, L, scratch, s, st);
        if (st != LV_OK)
            return st;
        auto k = raycast_warp_tiles_kernel<DT, F, EDGE, LA>;
        const uint32_t tiles =
            ((V.W + L.tile_w - 1) / L.tile_w) * ((V.H + L.tile_h - 1) / L.tile_h);
        const uint32_t grid =
            std::max(1u, std::min(resident_ctas(ctx, k, 128, 0), (tiles + 3) / 4));
        k<<<grid, 128, 0, s>>>(V, L.tile_w, L.tile_h, order);
        LV_CUDA(ctx, cudaGetLastError());
        return LV_OK;
    }
    if (L.kind == LV_LAUNCH_TILE_GRID)
        return tiles_dispatch<DT, F, EDGE, LA>(ctx, V, L, s, scratch);
    if (L.kind == LV_LAUNCH_TILE_QUEUE)
    {
        lv_status st = LV_OK;
        const uint32_t* order = frame_order(ctx, V, L, scratch, s, st);
        if (st != LV_OK)
            return st;
        auto k = raycast_queue_kernel<DT, F, EDGE, LA>;
        const uint32_t threads = L.tile_w * L.tile_h;
        const uint32_t tiles =
            ((V.W + L.tile_w - 1) / L.tile_w) * ((V.H + L.tile_h - 1) / L.tile_h);
        const uint32_t grid =
            std::max(1u, std::min(resident_ctas(ctx, k, int(threads), 0), tiles));
        k<<<grid, threads, 0, s>>>(V, L.tile_w, L.tile_h, order);
        LV_CUDA(ctx, cudaGetLastError());
        return LV_OK;
    }
    const dim3 block(L.tile_w, L.tile_h);
    const dim3 grid((V.W + block.x - 1) / block.x, (V.H + block.y - 1) / block.y);
    raycast_kernel<DT, F, EDGE, LA><<<grid, block, 0, s>>>(V);
    LV_CUDA(ctx, cudaGetLastError());
    return LV_OK;
}

/* One CTA per tile for bricks of NX x NX voxels in x and y, the pitches as
 * immediates: 34, 66 and 130 are the 32^3, 64^3 and 128^3 bricks with an
 * overlap of 1. LA: one-sample look-ahead. */
template <int DT, int F, int NX, int LA>
lv_status tiles_nx_dispatch(lv_ctx* ctx, const RayView& V, const lv_render_launch& L,
                            cudaStream_t s, uint8_t* scratch)
{
    lv_status st = LV_OK;
    const uint32_t* order = frame_order(ctx, V, L, scratch, s, st);
    if (st != LV_OK)
        return st;
    const uint32_t tiles = ((V.W + L.tile_w - 1) / L.tile_w) * ((V.H + L.tile_h - 1) / L.tile_h);
    raycast_tiles_kernel<DT, F, NX, LA><<<tiles, L.tile_w * L.tile_h, 0, s>>>(V, L.tile_w,
                                                                            L.tile_h, order);
    LV_CUDA(ctx, cudaGetLastError());
    return LV_OK;
}

template <int DT, int F, int EDGE>
lv_status plain_dispatch(lv_ctx* ctx, const RayView& V, const lv_render_launch& L,
                         cudaStream_t s, uint8_t* scratch)
{
    if (EDGE == 0 && F == LV_FILTER_TRILINEAR && L.kind == LV_LAUNCH_TILE_GRID &&
        V.N[0] == V.N[1] && (V.N[0] == 66 || V.N[0] == 34 || V.N[0] == 130) &&
        fixed_pitch_layout(V))
    {
        if (L.lookahead)
            return V.N[0] == 66   ? tiles_nx_dispatch<DT, F, 66, 1>(ctx, V, L, s, scratch)
                   : V.N[0] == 34 ? tiles_nx_dispatch<DT, F, 34, 1>(ctx, V, L, s, scratch)
                                  : tiles_nx_dispatch<DT, F, 130, 1>(ctx, V, L, s, scratch);
        return V.N[0] == 66   ? tiles_nx_dispatch<DT, F, 66, 0>(ctx, V, L, s, scratch)
               : V.N[0] == 34 ? tiles_nx_dispatch<DT, F, 34, 0>(ctx, V, L, s, scratch)
                              : tiles_nx_dispatch<DT, F, 130, 0>(ctx, V, L, s, scratch);
    }
    if (L.kind == LV_LAUNCH_WARP_REFILL)
        return refill_dispatch<DT, F, EDGE>(ctx, V, L, s);
    if (L.lookahead)
        return plain_dispatch_la<DT, F, EDGE, 1>(ctx, V, L, s, scratch);
    return plain_dispatch_la<DT, F, EDGE, 0>(ctx, V, L, s, scratch);
}

/* combination index (batch_group): 0..7 dtype (u8 0 / u16 1), filter,
 * edge; 8..13 trilinear bricks of pitch 34 / 66 / 130 (u8, then u16) */
template <int TFS>
lv_status persistent_by_index(int idx, lv_ctx* ctx, const RayView* d, const TileQueue& Q,
                              uint32_t ctas, size_t smem, cudaStream_t s)
{
    switch (idx)
    {
    case 8: return persistent_dispatch<LV_DT_UINT8, 1, TFS, 34>(ctx, d, Q, ctas, smem, s);
    case 9: return persistent_dispatch<LV_DT_UINT8, 1, TFS, 66>(ctx, d, Q, ctas, smem, s);
    case 10: return persistent_dispatch<LV_DT_UINT8, 1, TFS, 130>(ctx, d, Q, ctas, smem, s);
    case 11: return persistent_dispatch<LV_DT_UINT16, 1, TFS, 34>(ctx, d, Q, ctas, smem, s);
    case 12: return persistent_dispatch<LV_DT_UINT16, 1, TFS, 66>(ctx, d, Q, ctas, smem, s);
    case 13: return persistent_dispatch<LV_DT_UINT16, 1, TFS, 130>(ctx, d, Q, ctas, smem, s);
    case 0: return persistent_dispatch<LV_DT_UINT8, 0, TFS, 0>(ctx, d, Q, ctas, smem, s);
    case 1: return persistent_dispatch<LV_DT_UINT8, 0, TFS, 1>(ctx, d, Q, ctas, smem, s);
    case 2: return persistent_dispatch<LV_DT_UINT8, 1, TFS, 0>(ctx, d, Q, ctas, smem, s);
    case 3: return persistent_dispatch<LV_DT_UINT8, 1, TFS, 1>(ctx, d, Q, ctas, smem, s);
    case 4: return persistent_dispatch<LV_DT_UINT16, 0, TFS, 0>(ctx, d, Q, ctas, smem, s);
    case 5: return persistent_dispatch<LV_DT_UINT16, 0, TFS, 1>(ctx, d, Q, ctas, smem, s);
    case 6: return persistent_dispatch<LV_DT_UINT16, 1, TFS, 0>(ctx, d, Q, ctas, smem, s);
    default: return persistent_dispatch<LV_DT_UINT16, 1, TFS, 1>(ctx, d, Q, ctas, smem, s);
    }
}

lv_status refill_views_by_index(int idx, lv_ctx* ctx, const RayView* d, const TileQueue& Q,
                                uint32_t ctas, uint32_t checks, cudaStream_t s)
{
    /* the fixed-pitch groups take the general trilinear kernels */
    if (idx >= 8 && idx <= 10)
        idx = 2;
    else if (idx >= 11 && idx <= 13)
        idx = 6;
    switch (idx)
    {
    case 0: return refill_views_dispatch<LV_DT_UINT8, 0, 0>(ctx, d, Q, ctas, checks, s);
    case 1: return refill_views_dispatch<LV_DT_UINT8, 0, 1>(ctx, d, Q, ctas, checks, s);
    case 2: return refill_views_dispatch<LV_DT_UINT8, 1, 0>(ctx, d, Q, ctas, checks, s);
    case 3: return refill_views_dispatch<LV_DT_UINT8, 1, 1>(ctx, d, Q, ctas, checks, s);
    case 4: return refill_views_dispatch<LV_DT_UINT16, 0, 0>(ctx, d, Q, ctas, checks, s);
    case 5: return refill_views_dispatch<LV_DT_UINT16, 0, 1>(ctx, d, Q, ctas, checks, s);
    case 6: return refill_views_dispatch<LV_DT_UINT16, 1, 0>(ctx, d, Q, ctas, checks, s);
    default: return refill_views_dispatch<LV_DT_UINT16, 1, 1>(ctx, d, Q, ctas, checks, s);
    }
}
} // namespace

size_t tile_order_bytes(const RayView& V, const lv_render_launch& L)
{
    return order_bytes_of(V, L);
}

int batch_group(const RayView& V)
{
    const int v = kernel_variant(V.dtype, V.filter, V.edge);
    if (v >= 8 || V.filter != LV_FILTER_TRILINEAR || V.edge != 0 || V.N[0] != V.N[1] ||
        !fixed_pitch_layout(V))
        return v < 8 ? v : kBatchGroups + v;
    const int pitch = V.N[0] == 34 ? 0 : V.N[0] == 66 ? 1 : V.N[0] == 130 ? 2 : -1;
    if (pitch < 0)
        return v;
    return 8 + (V.dtype == LV_DT_UINT16 ? 3 : 0) + pitch;
}

/* 0..7: uint8 / uint16 x filter x edge; 8..11: the other voxel types x
 * filter x edge */
int kernel_variant(uint32_t dtype, uint32_t filter, uint32_t edge)
{
    const int fe = (filter == LV_FILTER_TRILINEAR ? 2 : 0) + (edge ? 1 : 0);
    if (dtype != LV_DT_UINT8 && dtype != LV_DT_UINT16)
        return 8 + fe;
    return (dtype == LV_DT_UINT16 ? 4 : 0) + fe;
}

lv_status launch_raycast(lv_ctx* ctx, const RayView& V, cudaStream_t s)
{
    if (V.dtype > LV_DT_INT32)
        return fail(ctx, LV_EINVAL, "unknown voxel type");
    /* the ray-cast kernels derive the samples per ray themselves */
    return launch_view_raycast(ctx, V, ctx->launch, nullptr, s);
}

lv_status launch_view_raycast(lv_ctx* ctx, const RayView& V, const lv_render_launch& L,
                              uint8_t* order_scratch, cudaStream_t s)
{
    switch (kernel_variant(V.dtype, V.filter, V.edge))
    {
    case 8: return any_type_dispatch<0, 0>(ctx, V, L, s, order_scratch);
    case 9: return any_type_dispatch<0, 1>(ctx, V, L, s, order_scratch);
    case 10: return any_type_dispatch<1, 0>(ctx, V, L, s, order_scratch);
    case 11: return any_type_dispatch<1, 1>(ctx, V, L, s, order_scratch);
    case 0: return plain_dispatch<LV_DT_UINT8, 0, 0>(ctx, V, L, s, order_scratch);
    case 1: return plain_dispatch<LV_DT_UINT8, 0, 1>(ctx, V, L, s, order_scratch);
    case 2: return plain_dispatch<LV_DT_UINT8, 1, 0>(ctx, V, L, s, order_scratch);
    case 3: return plain_dispatch<LV_DT_UINT8, 1, 1>(ctx, V, L, s, order_scratch);
    case 4: return plain_dispatch<LV_DT_UINT16, 0, 0>(ctx, V, L, s, order_scratch);
    case 5: return plain_dispatch<LV_DT_UINT16, 0, 1>(ctx, V, L, s, order_scratch);
    case 6: return plain_dispatch<LV_DT_UINT16, 1, 0>(ctx, V, L, s, order_scratch);
    default: return plain_dispatch<LV_DT_UINT16, 1, 1>(ctx, V, L, s, order_scratch);
    }
}

lv_status launch_views_pipeline(lv_ctx* ctx, const ResolveView* d_resolve,
                                const RayView* d_rays, uint32_t n, cudaStream_t s)
{
    resolve_views_kernel<<<dim3(8, n), 256, 0, s>>>(d_resolve);
    prune_views_kernel<<<dim3(8, n), 256, 0, s>>>(d_resolve);
    leaf_fill_views_kernel<<<dim3(16, n), 256, 0, s>>>(d_resolve);
    step_views_kernel<<<(n + 127) / 128, 128, 0, s>>>(d_rays, n);
    LV_CUDA(ctx, cudaGetLastError());
    return LV_OK;
}

lv_status launch_batch_order(lv_ctx* ctx, const RayView* d_rays, const TileQueue& Q,
                             uint32_t max_items, uint8_t* keys, uint32_t* hist,
                             uint32_t* order, cudaStream_t s)
{
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const uint32_t blocks =
        std::max(1u, std::min((max_items + 255) / 256, uint32_t(sms) * 4u));
    LV_CUDA(ctx, cudaMemsetAsync(hist, 0, 2 * kTileBuckets * sizeof(uint32_t), s));
    batch_key_kernel<<<blocks, 256, 0, s>>>(d_rays, Q, keys, hist);
    batch_order_kernel<<<blocks, 256, 0, s>>>(Q, keys, hist, order);
    LV_CUDA(ctx, cudaGetLastError());
    return LV_OK;
}

lv_status launch_persistent(lv_ctx* ctx, int variant, const lv_batch_config& cfg,
                            const RayView* d_rays, const TileQueue& Q, uint32_t tfn_max,
                            cudaStream_t s)
{
    if (cfg.queue == LV_QUEUE_WARP_REFILL)
        return refill_views_by_index(variant, ctx, d_rays, Q, cfg.ctas_per_sm,
                                     cfg.samples_per_check, s);
    const size_t smem = cfg.tf_shared ? size_t(tfn_max) * 2 * sizeof(float4) : 0;
    if (cfg.tf_shared)
        return persistent_by_index<1>(variant, ctx, d_rays, Q, cfg.ctas_per_sm, smem, s);
    return persistent_by_index<0>(variant, ctx, d_rays, Q, cfg.ctas_per_sm, smem, s);
}

} // namespace lv

extern "C" lv_status lv_frame_to_rgba8(lv_ctx* ctx, const float* d_rgba,
                                       uint32_t width, uint32_t height,
                                       uint8_t* d_out, void* stream)
{
    using namespace lv;
    if (!ctx || (!d_rgba && width * height) || (!d_out && width * height))
        return fail(ctx, LV_EINVAL, "null argument");
    const uint64_t n = uint64_t(width) * height;
    if (n == 0)
        return LV_OK;
    LV_CUDA(ctx, cudaSetDevice(ctx->device));
    const uint32_t blocks = uint32_t(std::min<uint64_t>((n + 255) / 256, 4096));
    to_rgba8_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<const float4*>(d_rgba), reinterpret_cast<uchar4*>(d_out), n);
    LV_CUDA(ctx, cudaGetLastError());
    return LV_OK;
}
