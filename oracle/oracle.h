/*
 * Livre hot-path oracle: a CPU restatement of the reference's LOD selection,
 * volume-information derivation, transfer function and ray-cast shader math.
 *
 * TEST INFRASTRUCTURE ONLY. The product (livre_gb300/, include/livre_gb300.h)
 * never links, loads or calls this library; only tests/, the smoke check in
 * __graft_entry__.py and the CPU-baseline leg of bench.py do, and only as the
 * checker / CPU baseline.
 *
 * Parity status:
 *  - LOD selection (FP32): pinned by the reference's golden NodeId sets in
 *    tests/data/lodSelection.cpp:70-207 (8 cases).
 *  - fillRegularVolumeInfo: pinned by tests/data/volumeInformation.cpp:57-106
 *    and tests/data/dataSource.cpp:39-64.
 *  - Default transfer function / LUT quantisation: pinned by
 *    tests/core/transferFunction.cpp:53-72 and tests/core/tf_f.1dt.
 *  - Ray cast (FP64 shading, FP32 ray geometry): parity unpinned against the
 *    reference (no reference test pins shader pixels; the GLSL shader cannot
 *    run without a graphics API). It restates livre/eq/render/shaders/
 *    fragRayCast.glsl:72-207 and is cross-checked against its own per-brick
 *    transcription of the shader (mode OR_MODE_SHADER).
 */
#ifndef LIVRE_ORACLE_H
#define LIVRE_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Derived volume description (VolumeInformation after fillRegularVolumeInfo,
 * livre/data/VolumeInformation.h:42-111). */
typedef struct
{
    uint32_t voxels[3];
    uint32_t max_block[3]; /* maximumBlockSize (block + 2 * overlap) */
    uint32_t overlap[3];
    float wspv;            /* worldSpacePerVoxel */
    float world_size[3];
    uint32_t depth;        /* rootNode depth */
    uint32_t root_blocks[3];
} or_volume;

/* livre/data/DataSourcePlugin.cpp:73-95. Returns 0 on success. */
int or_fill_regular_volume_info(or_volume* vol);

/* livre/data/DataSourcePlugin.cpp:40-71 + LODNode.cpp:30-64: the FP32 world
 * box of a node, {minx, miny, minz, maxx, maxy, maxz}. */
void or_node_world_box(const or_volume* vol, uint64_t node_id, float box[6]);

/* livre/data/NodeId.cpp:92-114 (children order x outer, z inner). */
void or_node_children(uint64_t node_id, uint64_t out[8]);

/* Frustum-derived constants (livre/data/Frustum.cpp:24-76 with the vmmlib
 * Frustumf / FrustumCullerf math restated). Matrices are column-major. */
typedef struct
{
    float inv_mv[16];
    float inv_p[16];
    float left, right, bottom, top, nearp, farp;
    float planes[6][4]; /* left, right, bottom, top, near, far */
    float eye[3];
    float dir[3];
} or_frustum;

int or_frustum_setup(const float mv[16], const float proj[16], or_frustum* f);

/* DFS LOD selection: DFSTraversal.cpp:63-76 + SelectVisibles.cpp:45-131.
 * Writes the visible ids in DFS order after the range post-filter.
 * Returns 0, or -1 if capacity is too small (n_out still holds the count). */
int or_select_visible(const or_volume* vol, const float mv[16],
                      const float proj[16], uint32_t window_height, float sse,
                      uint32_t min_lod, uint32_t max_lod, const float range[2],
                      const float* clip_planes, uint32_t n_clip,
                      uint32_t time_step, uint64_t* out, uint32_t capacity,
                      uint32_t* n_out, uint64_t* n_visited);

/* Default transfer function (TransferFunction1D.cpp:56-90), 256 RGBA floats. */
void or_default_tf(float rgba[256 * 4]);
/* getLUT (TransferFunction1D.cpp:92-107): truncating x * 255 to uint8. */
void or_tf_lut(const float* rgba, uint32_t n, uint8_t* lut);

/* Synthetic blob volume: sum of isotropic Gaussian blobs (cut off at 6 sigma)
 * plus optional integer noise, quantised to uint8 / uint16. Every float
 * operation is a single IEEE round-to-nearest op so the CUDA generator
 * produces identical bytes. */
typedef struct
{
    uint32_t n_blobs;
    uint32_t noise;   /* half-width of the integer noise, 0 = none */
    uint32_t dtype;   /* 1 = uint8, 2 = uint16 */
    uint64_t seed;
} or_blob_params;

/* Fills one brick (max_block voxels per axis, x fastest) of node_id. */
int or_blob_brick(const or_volume* vol, const or_blob_params* bp,
                  uint64_t node_id, void* out);
/* The blob function itself at a point given in finest-level voxel units. */
float or_blob_value(const or_volume* vol, const or_blob_params* bp, float x,
                    float y, float z);
float or_exp_neg(float x);

/* Procedural fBm volume (the out-of-core workload): improved Perlin noise
 * (Perlin 2002) summed over octaves, the permutation a SplitMix64-seeded
 * Fisher-Yates shuffle, [-1, 1] mapped to the voxel type's range. Every
 * float operation is a single IEEE round-to-nearest op in a fixed order
 * (built without contraction) so the device generator produces identical
 * bytes. Parity unpinned: no reference test or golden vector covers it; it
 * is the synthetic input of the 8192^3 uint16 workload. */
typedef struct
{
    uint64_t seed;
    uint32_t octaves;
    float lacunarity, gain, frequency;
    uint32_t dtype; /* 1 = uint8, 2 = uint16 */
} or_fbm_params;

int or_fbm_brick(const or_volume* vol, const or_fbm_params* fp, uint64_t node_id,
                 void* out);
/* The noise field itself (one octave) at a point, for spot checks. */
float or_perlin(uint64_t seed, float x, float y, float z);

/* Ray cast. */
enum
{
    OR_MODE_PER_RAY = 0, /* samples on the global grid, per-ray brick order */
    OR_MODE_SHADER = 1,  /* per-brick shader loop, DistanceOperator order */
    OR_ACCUMULATE = 0x100, /* flag: rays start from the colour in `out` */
    OR_QUANT_WEIGHTS = 0x200 /* flag (per-ray mode): trilinear weights rounded
                                to 8 fractional bits, the fixed-point weights of
                                a texture unit's linear filter; measures what
                                hardware filtering would cost, nothing renders
                                with it */
};

typedef struct
{
    float mv[16];
    float proj[16];
    uint32_t width, height;
    uint32_t n_samples;      /* samples per world unit: step = 1 / n_samples */
    float alpha_correction;  /* maxSamplesPerRay / nSamplesPerRay */
    float early_exit;        /* 0.999 in the reference shader */
    float range_lo, range_hi;/* dataSourceRange */
    uint32_t filter;         /* 0 nearest, 1 trilinear */
    uint32_t n_clip;
    float clip[6][4];
} or_view;

/* Renders the set of bricks `node_ids` (the rendering set: a partition of
 * the visible region; when an id and one of its ancestors are both present
 * the ancestor wins, as RenderingSetGeneratorFilter.cpp:51-79 does).
 * bricks: n_nodes bricks of max_block^3 voxels (x fastest), dtype an lv_dtype
 * code (0 float, 1 uint8, 2 uint16, 3 uint32, 4 int8, 5 int16, 6 int32).
 * out_rgba: width*height*4 doubles, row y=0 is the bottom row.
 * n_threads <= 0 uses every hardware thread. */
int or_raycast(const or_volume* vol, uint32_t dtype, const uint64_t* node_ids,
               uint32_t n_nodes, const void* bricks, const float* tf_rgba,
               uint32_t tf_n, const or_view* view, int mode, int n_threads,
               uint32_t row_begin, uint32_t row_end, double* out_rgba,
               uint64_t* n_samples_out);

/* Per-pixel diagnostics of a ray cast (either pointer may be null; both
 * hold width*height entries, rows outside [row_begin, row_end) untouched).
 * px_samples: samples composited on the pixel's ray.
 * px_flags (shader mode only; 0 in per-ray mode): for each brick with at
 * least one sample, its first sample's index on the ray's global grid
 * (round((t - tnearGlobal) * nSamples)) against the last index of the brick
 * composited before it:
 *   OR_PX_DUPLICATE: equal, i.e. both bricks sampled the grid point on
 *     their shared face (the per-brick snapping of fragRayCast.glsl:142-147
 *     evaluated on each side of the face);
 *   OR_PX_INVERTED: smaller, i.e. a brick nearer the eye along the ray was
 *     composited after a farther one (the brick-centre distance order of
 *     RayCastRenderer.cpp:57-81 is not the ray's order there);
 *   OR_PX_GAP: larger by more than one while the previous brick's exit and
 *     this brick's entry parameters are equal (a face grid point neither
 *     brick sampled). */
#define OR_PX_DUPLICATE 1u
#define OR_PX_INVERTED 2u
#define OR_PX_GAP 4u
int or_raycast_px(const or_volume* vol, uint32_t dtype, const uint64_t* node_ids,
                  uint32_t n_nodes, const void* bricks, const float* tf_rgba,
                  uint32_t tf_n, const or_view* view, int mode, int n_threads,
                  uint32_t row_begin, uint32_t row_end, double* out_rgba,
                  uint64_t* n_samples_out, uint32_t* px_samples, uint8_t* px_flags);

#ifdef __cplusplus
}
#endif
#endif
