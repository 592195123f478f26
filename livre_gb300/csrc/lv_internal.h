/*
 * Internal device/host structures of the livre_gb300 runtime.
 *
 * NodeId packing follows livre::NodeId (livre/data/NodeId.h:34-49,
 * livre/data/types.h:80-93): bits [0,4) level, [4,18) x, [18,32) y,
 * [32,46) z, [46,64) time step; all ones = invalid.
 */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "livre_gb300.h"

#define LV_HD __host__ __device__ __forceinline__

namespace lv
{
constexpr uint32_t kMaxLevels = 15;
constexpr uint32_t kLeafEmpty = 0xFFFFFFFFu;
constexpr uint32_t kLeafSlotBits = 27;
constexpr uint32_t kLeafSlotMask = (1u << kLeafSlotBits) - 1u;
constexpr uint64_t kInvalidNode = ~0ull;
/* Pool addresses are stored as 1 KiB units (27 bits: 128 GiB). */
constexpr uint64_t kSlotUnit = 1024;

/* Brick layout in the pool for uint8 bricks of kQuadMinRow to kQuadMaxRow
 * voxels per row: voxel quads. Element i of a brick (the voxels in
 * x-fastest order) is 32 bits: voxel i in byte 0, its +x neighbour in byte
 * 1, its +y neighbour in byte 2 and its +x+y neighbour in byte 3 (a
 * neighbour past the end of a row or slice is the voxel itself), so a
 * trilinear sample's eight voxels are two aligned 32-bit loads (slices z and
 * z + 1) instead of eight byte loads. A single voxel is the element's byte
 * 0. Four times the bytes per brick. Smaller uint8 bricks and the other
 * voxel types keep one voxel per element (on the 256^3 / 32^3-brick
 * workload, whose frame time is its longest rays' chains, wider elements
 * measured slower). */
constexpr uint32_t kQuadMinRow = 64;
constexpr uint32_t kQuadMaxRow = 1024;
__host__ __device__ constexpr bool quad_layout(uint32_t dtype, uint32_t row_voxels)
{
    return dtype == LV_DT_UINT8 && row_voxels >= kQuadMinRow && row_voxels <= kQuadMaxRow;
}

LV_HD uint32_t nid_level(uint64_t id) { return uint32_t(id & 0xFu); }
LV_HD uint32_t nid_x(uint64_t id) { return uint32_t((id >> 4) & 0x3FFFu); }
LV_HD uint32_t nid_y(uint64_t id) { return uint32_t((id >> 18) & 0x3FFFu); }
LV_HD uint32_t nid_z(uint64_t id) { return uint32_t((id >> 32) & 0x3FFFu); }
LV_HD uint32_t nid_t(uint64_t id) { return uint32_t(id >> 46); }
LV_HD uint64_t nid_make(uint32_t level, uint32_t x, uint32_t y, uint32_t z,
                        uint32_t t)
{
    return uint64_t(level & 0xFu) | (uint64_t(x & 0x3FFFu) << 4) |
           (uint64_t(y & 0x3FFFu) << 18) | (uint64_t(z & 0x3FFFu) << 32) |
           (uint64_t(t & 0x3FFFFu) << 46);
}

/* Per-view constants of the LOD selection (derived on the host from
 * Frustum(MV, P) and the SelectVisibles arguments). */
struct LodView
{
    float planes[6][4];  /* culler planes: left right bottom top near far */
    float eye_near[3];   /* eye - dir * near (SelectVisibles.cpp:88-89) */
    float nearp;         /* frustum near limit */
    float wspp;          /* (top - bottom) / windowHeight */
    float sse;
    float world_size[3];
    float half[3];       /* world_size * 0.5f */
    float clip[6][4];
    uint32_t n_clip;
    uint32_t min_lod, max_lod, depth;
    uint32_t root_blocks[3];
    uint32_t block[3];   /* maximumBlockSize - 2 * overlap */
    uint32_t time_step;
    uint32_t root_offset; /* first root of this view in the level-0 frontier */
    uint32_t capacity;    /* of out_ids */
    uint64_t* out_ids;
    uint32_t* result;     /* LV_SELECT_RESULT_WORDS */
};

/* Voxel-type template argument of the ray-cast kernels for the types other
 * than uint8 and uint16 (int8, int16, uint32, int32, float), read through a
 * run-time switch on RayView::dtype. */
constexpr int kDtAny = -1;

/* Per-view constants of the ray cast. */
struct RayView
{
    float inv_p[16];
    float inv_mv[16];
    float eye[3];
    float nearp;
    float gmin[3], gmax[3], gscale[3];
    float goff[3];    /* half world size * gscale: f = fma(p, gscale, goff) */
    float clip[6][4];
    uint32_t n_clip;
    uint32_t dims[3]; /* leaf grid (finest level) */
    uint32_t Lf;      /* finest level = depth - 1 */
    uint32_t N[3], B[3], O[3];
    uint32_t dtype;   /* lv_dtype */
    uint32_t bpv;     /* bytes per voxel */
    uint32_t filter;
    uint32_t edge;    /* 1: some overlap is 0, clamp every trilinear tap */
    uint32_t quads;   /* bricks stored as voxel quads (quad_layout) */
    float dmul, dadd; /* density = value * dmul + dadd */
    float tf_mul, tf_add; /* TF texel coordinate = value * tf_mul + tf_add
                             = density * tfn - 0.5 */
    float tf_last;        /* tfn - 1 */
    uint32_t accumulate;  /* 1: rays start from the colour already in out (a
                             later pass of a multi-pass frame) */
    uint32_t skip_if_missing; /* 1: a synchronous frame's first ray cast, queued
                                 before its miss count reached the host: it
                                 renders nothing if the residency pass counted
                                 misses (the host streams them and renders the
                                 frame again) */
    uint32_t max_base;    /* last trilinear base voxel of a brick:
                             (N2-2)*N1*N0 + (N1-2)*N0 + N0-2 */
    float early;
    uint32_t W, H;          /* pixels rendered: the rect (tiles cover these) */
    uint32_t x0, y0;        /* the rect's corner in the frame */
    uint32_t FW, FH;        /* the frame (ray directions, output rows) */
    uint32_t cull[4];       /* frame pixels [cull[0], cull[2]) x [cull[1], cull[3]):
                               a conservative bound of the pixels whose ray can
                               reach the volume's box; the others start and end
                               with no sample */
    uint32_t samples_fixed; /* 0 = policy */
    uint32_t step_policy;
    uint32_t max_voxel_dim;
    uint32_t depth;
    const uint32_t* leaf;
    const uint8_t* pool; /* brick = pool + slot * kSlotUnit */
    uint32_t pool_units;  /* arena size in kSlotUnit units */
    uint32_t brick_units; /* units one brick of this volume occupies */
    const float4* tf; /* tfn (value, next - value) pairs */
    uint32_t tfn;
    float4* out;
    uint32_t* counters; /* FrameCounters */
};

/* Device counters of one frame of one view. */
enum FrameCounter
{
    FC_RENDERED = 0,      /* rendering-set entries */
    FC_AVAILABLE = 1,
    FC_NOT_AVAILABLE = 2,
    FC_MISSING = 3,       /* entries appended to the missing list */
    FC_MAX_LEVEL = 4,     /* finest level rendered, +1 (0 = none) */
    FC_SAMPLES_PER_RAY = 5,
    FC_SAMPLES_LO = 6,    /* 64-bit composited-sample counter */
    FC_SAMPLES_HI = 7,
    FC_ERROR = 8,         /* nonzero: an index check failed in a kernel */
    FC_KEPT = 9,          /* rendering-set entries left after dropping the
                             ones with an ancestor in the set */
    FC_QUEUE = 10,        /* tile queue head of the single-view ray cast */
    FC_WORDS = 16
};

/* Per-view inputs of the residency pass. */
struct ResolveView
{
    const uint64_t* visible;  /* visible ids of the view */
    const uint32_t* n_visible_ptr; /* LV_SEL_WRITTEN word of the selection */
    const int32_t* node_table;     /* slot unit per node (-1 = not resident) */
    uint32_t* node_stamp;          /* last frame a node was rendered (in use) */
    uint32_t* view_stamp;          /* per-view stamps: rendering-set membership */
    uint32_t frame;                /* stamp written to node_stamp */
    uint32_t view_frame;           /* stamp written to view_stamp */
    uint32_t depth;
    uint32_t root_blocks[3];
    uint64_t level_offset[kMaxLevels + 1];
    uint32_t synchronous;     /* no ancestor fallback */
    uint64_t* render_ids;     /* rendering set: ids */
    uint32_t* render_slots;   /* rendering set: slot */
    uint32_t render_capacity;
    uint64_t* missing;        /* missing ids */
    uint32_t missing_capacity;
    uint32_t* counters;       /* FrameCounters */
    uint32_t* leaf;           /* leaf grid */
    uint32_t dims[3];
    uint32_t Lf;
    uint64_t n_nodes;         /* entries of node_table / stamps */
};

/* Work queue of the persistent ray-cast kernel: the views of one voxel
 * type / filter group and the prefix sums of their tile counts. */
struct TileQueue
{
    const uint32_t* view_ids;   /* n_views entries: index into the RayView array */
    const uint32_t* tile_start; /* n_views + 1 prefix sums */
    const uint32_t* n_views;    /* device word: views of this group (per launch) */
    uint32_t tile_w, tile_h;
    uint32_t* head;             /* zeroed before the launch */
    const uint32_t* order;      /* nullable: item k of the queue is work item
                                   order[k] (longest first) */
    unsigned long long* clock;  /* [first CTA start, last CTA end] in ns (%globaltimer) */
};

LV_HD uint64_t node_index(const uint64_t* level_offset,
                          const uint32_t* root_blocks, uint64_t id)
{
    const uint32_t L = nid_level(id);
    const uint64_t by = uint64_t(root_blocks[1]) << L;
    const uint64_t bz = uint64_t(root_blocks[2]) << L;
    return level_offset[L] +
           (uint64_t(nid_x(id)) * by + nid_y(id)) * bz + nid_z(id);
}

} // namespace lv

/* Host-side helpers implemented in the .cu files. */
namespace lv
{
void frustum_setup(const float* mv, const float* p, float inv_mv[16],
                   float inv_p[16], float limits[6], float planes[6][4],
                   float eye[3], float dir[3], bool* ok);
}
