/*
 * livre_gb300: GB300-native (sm_103a) implementation of Livre's rendering hot
 * path behind a C ABI: octree LOD + frustum brick selection, a device-resident
 * HBM brick pool with an LRU page table fed from host memory, and
 * front-to-back ray-cast compositing with a 1D RGBA transfer function.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, and returns
 * an lv_status. Device buffers passed in (d_*) are CUDA device pointers owned
 * by the caller; `stream` is a cudaStream_t (NULL = legacy default stream).
 * The library owns the brick pool, page tables and transfer-function copies.
 * A context is used by one host thread at a time (or externally serialised).
 *
 * Reference interfaces (paths inside BlueBrain/Livre) are cited per entry.
 */
#ifndef LIVRE_GB300_H
#define LIVRE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LV_ABI_VERSION 1

typedef enum lv_status
{
    LV_OK = 0,
    LV_EINVAL = 1,    /* invalid argument */
    LV_ENOMEM = 2,    /* device/host allocation failed or capacity exceeded */
    LV_ETIMEDOUT = 3, /* a bounded device wait gave up */
    LV_EDEVICE = 4,   /* CUDA error */
    LV_ENOTFOUND = 5, /* data source returned no data for a node */
    LV_EAGAIN = 6     /* resource busy (pool full of bricks in use) */
} lv_status;

/* Voxel types, same order as livre::DataType (livre/data/VolumeInformation.h:31-41). */
typedef enum lv_dtype
{
    LV_DT_FLOAT = 0,
    LV_DT_UINT8 = 1,
    LV_DT_UINT16 = 2,
    LV_DT_UINT32 = 3,
    LV_DT_INT8 = 4,
    LV_DT_INT16 = 5,
    LV_DT_INT32 = 6
} lv_dtype;

/* livre::VolumeInformation (livre/data/VolumeInformation.h:42-111). The caller
 * fills voxels, max_block (maximumBlockSize = block + 2 * overlap), overlap,
 * dtype and comp_count; lv_fill_regular_volume_info derives the rest. */
typedef struct lv_volume_info
{
    uint32_t voxels[3];
    uint32_t max_block[3];
    uint32_t overlap[3];
    uint32_t dtype;
    uint32_t comp_count;
    float world_space_per_voxel;
    float world_size[3];
    uint32_t depth;          /* RootNode::getDepth() */
    uint32_t root_blocks[3]; /* RootNode::getBlockSize(0) */
} lv_volume_info;

/* Replaces livre::fillRegularVolumeInfo (livre/data/DataSourcePlugin.cpp:73-95). */
lv_status lv_fill_regular_volume_info(lv_volume_info* info);

/* livre::Frustum(modelView, projection) (livre/data/Frustum.h:46-47):
 * 4x4 matrices stored column-major like vmml::Matrix4f::array. */
typedef struct lv_camera
{
    float modelview[16];
    float projection[16];
} lv_camera;

/* Inputs of SelectVisibles (livre/data/SelectVisibles.h:44-47) as wired by
 * VisibleSetGeneratorFilter::execute (livre/lib/pipeline/
 * VisibleSetGeneratorFilter.cpp:40-66). */
typedef struct lv_lod_params
{
    uint32_t window_height;   /* pixel viewport height (vp[3]) */
    float screen_space_error; /* VolumeRendererParameters screen_space_error */
    uint32_t min_lod;
    uint32_t max_lod;
    float range[2];           /* sort-last data range, {0, 1} on one GPU */
    uint32_t time_step;
    uint32_t n_clip_planes;   /* <= 6; plane (n, d) keeps n.p + d >= 0 */
    float clip_planes[6][4];
} lv_lod_params;

/* Result words written by lv_select_visible into d_result[LV_SELECT_RESULT_WORDS]. */
enum
{
    LV_SEL_WRITTEN = 0,   /* ids written to d_out_ids (<= capacity) */
    LV_SEL_FOUND = 1,     /* visible ids found (after the range slice) */
    LV_SEL_VISITED = 2,   /* octree nodes visited */
    LV_SEL_MAX_LEVEL = 3, /* finest level among the visible ids */
    LV_SEL_OVERFLOW = 4,  /* 1: a traversal frontier overflowed; 2: the
                             single-launch selection's grid barrier gave up
                             waiting (the ids are unusable) */
    LV_SELECT_RESULT_WORDS = 8
};

typedef struct lv_ctx lv_ctx;
typedef struct lv_volume lv_volume;
typedef struct lv_tf lv_tf;

/* Context on one CUDA device. Not in the reference (GL context + caches of
 * livre/eq/Window.cpp:54-72 play this role). */
lv_status lv_ctx_create(int device, lv_ctx** out);
void lv_ctx_destroy(lv_ctx* ctx);
/* Last error message of this context ("" when none). */
const char* lv_last_error(const lv_ctx* ctx);
/* Library ABI version and the CUDA architecture it was built for. */
uint32_t lv_abi_version(void);

/* LOD selection on the device. Replaces DFSTraversal::traverse(rootNode,
 * SelectVisibles, timeStep) (livre/data/DFSTraversal.cpp:63-76 with
 * livre/data/SelectVisibles.cpp:45-131). The visible NodeIds are bit-exact to
 * the reference's FP32 selection; they are written level by level (the
 * reference's DFS order is restored only when the range slice needs it).
 * d_out_ids: capacity uint64 device slots; d_result: LV_SELECT_RESULT_WORDS
 * uint32 device words. Asynchronous on `stream`. Scratch (frontier queues) is
 * allocated by the context on first use and reused; lv_render's selection
 * shares it, and each waits for the other's earlier use whatever the
 * streams. */
lv_status lv_select_visible(lv_ctx* ctx, const lv_volume_info* vol,
                            const lv_camera* camera,
                            const lv_lod_params* params, uint64_t* d_out_ids,
                            uint32_t capacity, uint32_t* d_result,
                            void* stream);

/* The visible set of one view in host memory: lv_select_visible into the
 * context's own device buffer, then copied to `ids` (capacity uint64 host
 * slots) and `result` (LV_SELECT_RESULT_WORDS host words). Synchronous. The
 * output port "VisibleNodes" of VisibleSetGeneratorFilter::execute
 * (livre/lib/pipeline/VisibleSetGeneratorFilter.cpp:40-66), which
 * RenderPipeline::render hands to Renderer::render
 * (livre/lib/pipeline/RenderPipeline.cpp:92-158). */
lv_status lv_select_visible_host(lv_ctx* ctx, const lv_volume_info* vol,
                                 const lv_camera* camera,
                                 const lv_lod_params* params, uint64_t* ids,
                                 uint32_t capacity, uint32_t* result);

/* Test hook of the selection's failure path; no counterpart in the
 * reference (its CPU traversal has no barrier). The next single-view
 * selection that runs as one cooperative launch (lv_select_visible, or
 * lv_render's selection when the previous frame has finished) launches with
 * one CTA that never arrives at the grid barrier and a wait limit of `polls`
 * polls (64 ns sleeps) instead of 2^22: the other CTAs give up, the launch
 * returns, and the selection reports LV_SEL_OVERFLOW = 2 (lv_select_visible)
 * or error_flags 4 (lv_render). Selections of octrees whose widest level
 * fits one CTA (<= 256 nodes) run on one CTA and are not affected. polls:
 * 1 .. 2^22. */
lv_status lv_test_fail_grid_barrier(lv_ctx* ctx, uint32_t polls);

/* LOD selection that allocates nothing, for callers that cannot allocate
 * device memory (a host application whose own caching allocator owns the
 * GPU's memory, or a per-frame path that must not risk the device-wide
 * synchronisation of an allocation). No counterpart in the reference.
 * Same inputs and outputs as lv_select_visible, no context: it runs on the
 * current device, with its frontier queues in one fixed device array of the
 * library (about 6.3 MB, held by every GPU that loads the library until the
 * process exits). Limits: at most 262144 nodes per octree level (larger
 * volumes return LV_ENOMEM) and range {0, 1} only (LV_EINVAL otherwise).
 * The first call on a device does a one-time set-up (it looks up that
 * array's device address and the SM count); make that first call before any
 * stream capture on the device. With CUDA's lazy module loading the array is
 * reserved when the library's selection module first loads on a device (that
 * first call, or the first selection of lv_render / lv_select_visible): make
 * it before the application's allocator takes the GPU's memory. All calls
 * share the array and it keeps the last call's contents (each call clears
 * what must start at zero): calls whose work overlaps on the GPU race and
 * must be ordered by the caller. An error already pending on the calling
 * thread (cudaPeekAtLastError) returns LV_EDEVICE and is left in place. */
lv_status lv_select_visible_noalloc(const lv_volume_info* vol,
                                    const lv_camera* camera,
                                    const lv_lod_params* params,
                                    uint64_t* d_out_ids, uint32_t capacity,
                                    uint32_t* d_result, void* stream);

/* ---------------------------------------------------------- brick pool */

/* Device brick pool budget in bytes (VolumeRendererParameters
 * max_gpu_cache_memory, livre/lib/zeroeq/volumeRendererParameters.fbs:9;
 * Cache byte budget, livre/core/cache/Cache.cpp:41-96). Must be called before
 * the first volume is created. Default: 3072 MiB. */
lv_status lv_pool_configure(lv_ctx* ctx, size_t bytes);
/* Drops every resident brick (Cache::purge, livre/core/cache/Cache.cpp:186-192). */
lv_status lv_pool_purge(lv_ctx* ctx);
/* Brick layouts in the pool (no reference counterpart: the reference keeps
 * one texture per brick, TextureObject.cpp:76-120). */
enum
{
    LV_BRICKS_QUADS = 0,  /* default: uint8 bricks of 64 to 1024 voxels per
                             row stored as voxel quads (each voxel with its
                             +x, +y and +x+y neighbours in one 32-bit
                             element), so a trilinear sample reads two words
                             instead of eight bytes: four times the pool
                             bytes; on a 2048^3 volume of 64^3 bricks at
                             1920x1080, 0.232 ms of ray cast per frame
                             against 0.282 ms measured with one byte per
                             voxel; other bricks compact */
    LV_BRICKS_COMPACT = 1 /* one voxel per element for every brick: four
                             times as many large uint8 bricks per pool byte
                             (a server whose volumes' visible sets outgrow
                             the pool with quads) */
};
/* Brick layout of the pool; like lv_pool_configure, before the first volume
 * is created. */
lv_status lv_pool_set_brick_layout(lv_ctx* ctx, uint32_t layout);
/* Pool bytes one brick of a volume with this description occupies on ctx
 * (its brick layout; ctx NULL: the default layout), for sizing the pool
 * (TextureObject's texture size, livre/core/render/TextureObject.cpp:76-120,
 * in whole 1 KiB units). */
lv_status lv_brick_slot_bytes(const lv_ctx* ctx, const lv_volume_info* info, uint64_t* bytes);

/* livre::DataSourcePlugin::getData (livre/data/DataSourcePlugin.h:81) as a C
 * callback: fill `dst` (page-locked host memory, `bytes` long: the node's
 * (block + 2 * overlap)^3 voxels, x fastest) for `node_id` and return 0, or
 * return nonzero for a null MemoryUnitPtr. Called from the thread that
 * renders, one brick at a time (the reference's single upload thread,
 * livre/lib/pipeline/RenderPipeline.cpp:42), unless the volume's fetch
 * threads are raised. */
typedef int (*lv_get_data_fn)(void* user, uint64_t node_id, void* dst,
                              size_t bytes);

/* A volume whose bricks come from a data-source callback (plugin). */
lv_status lv_volume_create(lv_ctx* ctx, const lv_volume_info* info,
                           lv_get_data_fn get_data, void* user,
                           lv_volume** out);
/* Host threads that call the volume's get_data at once for a frame's missing
 * bricks (0: one per hardware thread, at most 64; default 1). Above 1 the
 * callback must be re-entrant. Each thread fills its own page-locked staging
 * buffer; a group's copies to the device overlap the next group's fetch.
 * LV_EINVAL for a volume that is not fed by a callback. */
lv_status lv_volume_set_fetch_threads(lv_volume* vol, uint32_t threads);
lv_status lv_volume_get_fetch_threads(const lv_volume* vol, uint32_t* threads);

/* Synthetic blob volume: sum of n_blobs isotropic Gaussians (centres uniform
 * in the volume, sigma U[8,32] voxels, amplitude U[0.3,1], cut off at
 * 6 sigma) plus integer noise U[-noise, noise], from `seed`. */
typedef struct lv_blob_desc
{
    uint32_t n_blobs;
    uint32_t noise;
    uint64_t seed;
} lv_blob_desc;

/* Where the bricks of a blob volume live before they are needed. */
enum
{
    LV_BLOB_DEVICE = 0, /* generated on the device, straight into the pool */
    LV_BLOB_HOST = 1    /* generated once into page-locked host memory and
                           streamed host->device on a miss */
};
lv_status lv_volume_create_blob(lv_ctx* ctx, const lv_volume_info* info,
                                const lv_blob_desc* blob, uint32_t placement,
                                lv_volume** out);
void lv_volume_destroy(lv_volume* vol);
/* The derived VolumeInformation of a volume. */
lv_status lv_volume_get_info(const lv_volume* vol, lv_volume_info* out);

/* Procedural fBm volume: `octaves` octaves of improved Perlin noise
 * (Perlin 2002) with the given lacunarity and gain, `frequency` noise
 * periods across the largest volume dimension, the permutation shuffled by
 * SplitMix64 draws from `seed`; [-1, 1] maps linearly to the full range of
 * the voxel type. */
typedef struct lv_fbm_params
{
    uint64_t seed;
    uint32_t octaves;
    float lacunarity, gain, frequency;
} lv_fbm_params;
enum
{
    LV_FBM_DEVICE = 0, /* generated on the device, straight into the pool */
    LV_FBM_HOST = 1    /* generated on the host when it misses (a
                          data-source callback, one brick per fetch thread,
                          host_threads of them: 0 = one per hardware
                          thread), then streamed host->device */
};
lv_status lv_volume_create_fbm(lv_ctx* ctx, const lv_volume_info* info,
                               const lv_fbm_params* params, uint32_t placement,
                               uint32_t host_threads, lv_volume** out);
/* One fBm brick (max_block voxels, x fastest) on the host, as a data-source
 * plugin's getData would produce it; no context or device needed. The device
 * generator produces the same bytes. */
lv_status lv_fbm_brick(const lv_volume_info* info, const lv_fbm_params* params,
                       uint64_t node_id, void* dst, uint32_t n_threads);
/* The same bricks for `n` node ids (host array) generated on the device into
 * d_out (n bricks, packed). Synchronous with `stream`. */
lv_status lv_fbm_generate(lv_ctx* ctx, const lv_volume_info* info,
                          const lv_fbm_params* params, const uint64_t* ids, uint32_t n,
                          void* d_out, void* stream);

/* Data sources registered at run time, tried by lv_volume_open before the
 * built-in ones in registration order: the plugin factory of the reference
 * (livre/data/DataSource.cpp:29-63), which a C++ plugin reaches through
 * lunchbox::PluginRegisterer (include/lunchbox/pluginRegisterer.h).
 * handles(user, uri) != 0 when the source opens `uri`; open fills the
 * volume description (fillRegularVolumeInfo applied) and the brick callback,
 * whose `source` pointer source_free releases with the volume. */
typedef int (*lv_source_handles_fn)(void* user, const char* uri);
typedef lv_status (*lv_source_open_fn)(void* user, const char* uri, lv_volume_info* info,
                                       lv_get_data_fn* get_data, void** source,
                                       void (**source_free)(void*));
lv_status lv_register_source(lv_source_handles_fn handles, lv_source_open_fn open, void* user,
                             const char* description);
lv_status lv_unregister_source(lv_source_handles_fn handles, lv_source_open_fn open);
/* The data source for `uri` without a context or device, as
 * livre::DataSource(uri) constructs it (livre/data/DataSource.cpp:29-56): a
 * registered source that handles `uri`, else a built-in one (mem://, raw://).
 * Fills the volume description and the brick callback; source_free(*source)
 * releases it. LV_EINVAL when no source handles `uri` or it fails to open. */
lv_status lv_source_open(const char* uri, lv_volume_info* info, lv_get_data_fn* get_data,
                         void** source, void (**source_free)(void*));
/* The description of the volume lv_source_open gives for `uri` (the source is
 * opened and closed again). */
lv_status lv_source_probe(const char* uri, lv_volume_info* info);
/* DataSource::loadPlugins (livre/data/DataSource.cpp:58-62): loads every
 * shared library ending in ".so" whose file name contains a match of the
 * regular expression `pattern` (NULL: "Livre.*Source"), found in the
 * ':'-separated directories `paths` (NULL: LD_LIBRARY_PATH). Their static
 * PluginRegisterer objects register their sources; the libraries stay loaded.
 * *n_loaded (may be NULL) counts the libraries newly loaded. A library that
 * fails to load is skipped, as the reference's factory does. */
lv_status lv_load_plugins(const char* paths, const char* pattern, uint32_t* n_loaded);
/* DataSource::getDescriptions (livre/data/DataSource.cpp:64-68): the
 * descriptions of the registered sources, then of the built-in ones, as one
 * NUL-terminated string; out = NULL asks for the size (with the NUL). */
lv_status lv_source_descriptions(char* out, size_t capacity, size_t* size);
/* DataSource::handles (livre/data/DataSource.cpp:70-74): 1 when a
 * registered or built-in source opens `uri`, else 0. */
int lv_source_handles(const char* uri);

/* A volume opened from a URI by the built-in data sources, like
 * livre::DataSource(uri) (livre/data/DataSource.cpp:29-63):
 *   mem://[#w,h,d,block][?datatype=T]   MemoryDataSource (constant bricks)
 *   raw://f.raw#x,y,z[,T]                RawDataSource (one brick)
 *   raw://f.nrrd[?output=T]              RawDataSource with an NRRD header
 * Unknown schemes return LV_EINVAL ("no data source handles ..."). */
lv_status lv_volume_open(lv_ctx* ctx, const char* uri, lv_volume** out);
/* DataSource::getData (livre/data/DataSource.cpp:101-111): the brick of
 * `node_id` into host memory `dst` (at least the brick's bytes); LV_ENOTFOUND
 * for invalid ids or a source that has no data for the node. */
lv_status lv_volume_get_data(lv_volume* vol, uint64_t node_id, void* dst,
                             size_t bytes);

/* Loads the bricks `ids` (host array) of `vol` into the pool now, evicting
 * the oldest resident bricks when it is full, like Cache::load<TextureObject>
 * (livre/core/cache/Cache.cpp:111-123) driven by DataUploadFilter::load
 * (livre/lib/pipeline/DataUploadFilter.cpp:45-77). Already resident ids are
 * hits and keep their place in the eviction order. Synchronous. */
lv_status lv_volume_load(lv_volume* vol, const uint64_t* ids, uint32_t n,
                         uint32_t* n_loaded);
/* Resident node ids of `vol` in eviction order (oldest load first), like
 * the LRU queue of livre/core/cache/Cache.cpp:41-96. */
lv_status lv_volume_resident(const lv_volume* vol, uint64_t* ids,
                             uint32_t capacity, uint32_t* n);

/* Generates blob bricks for `n` node ids (host array `ids`) into d_out (n
 * bricks of max_block^3 voxels, x fastest) on the device. */
lv_status lv_blob_generate(lv_ctx* ctx, const lv_volume_info* info,
                           const lv_blob_desc* blob, const uint64_t* ids,
                           uint32_t n, void* d_out, void* stream);

/* Value histograms of bricks `ids` (host array; loaded into the pool if
 * missing), replacing HistogramObject (livre/lib/cache/HistogramObject.cpp:
 * 30-224) and the accumulation of HistogramFilter::execute (livre/lib/
 * pipeline/HistogramFilter.cpp:78-149) for a full viewport. Only each brick's
 * own voxels count, weighted by (2^(depth-1-level))^3 finest voxels per voxel;
 * value v falls in bin floor((v - lo) * (n_bins - 1) / (hi - lo)) clamped to
 * the bins (bin = v for uint8, 256 bins over [0, 255]). per_brick (nullable):
 * n * n_bins host words; accumulated: n_bins host words. Synchronous. */
lv_status lv_histogram(lv_volume* vol, const uint64_t* ids, uint32_t n,
                       uint32_t n_bins, float range_lo, float range_hi,
                       uint64_t* per_brick, uint64_t* accumulated);

/* ------------------------------------------------------ transfer function */

/* A resident 1D RGBA transfer function of n float entries (host rgba, 4*n
 * floats). Replaces the GL_RGBA8 1D texture of
 * livre/eq/render/RayCastRenderer.cpp:175-193; sampled with linear filtering
 * and clamp-to-edge. */
lv_status lv_tf_create(lv_ctx* ctx, const float* rgba, uint32_t n,
                       lv_tf** out);
void lv_tf_destroy(lv_tf* tf);

/* ----------------------------------------------------------- rendering */

enum
{
    LV_FILTER_NEAREST = 0,
    LV_FILTER_TRILINEAR = 1
};
enum
{
    LV_STEP_REFERENCE = 0, /* max(maxVoxels >> (depth-1-L), 512) per unit
                              (livre/eq/render/RayCastRenderer.cpp:216-233) */
    LV_STEP_HALF_VOXEL = 1 /* 0.5 voxel of the finest rendered level */
};

typedef struct lv_render_desc
{
    lv_camera camera;
    uint32_t width, height;    /* pixel viewport */
    lv_lod_params lod;         /* window_height is taken from `height` if 0 */
    uint32_t samples_per_ray;  /* 0 = from step_policy */
    uint32_t step_policy;
    float early_exit;          /* 0.999 in fragRayCast.glsl:12 */
    uint32_t filter;
    float data_range[2];       /* dataSourceRange, used when hi > 0 and hi > lo,
                                  else the voxel type's range */
    uint32_t synchronous;      /* 1: stream every missing brick first
                                  (RenderPipeline::renderSync); 0: render the
                                  nearest resident ancestors and stream up to
                                  max_uploads misses (renderAsync) */
    uint32_t max_uploads;      /* async mode only; reference: 1 per frame */
    uint32_t rect[4];          /* {x, y, w, h}: render only these pixels of the
                                  width x height frame (a sort-first tile,
                                  Channel.cpp:234-281), writing them at their
                                  place in d_rgba and no others; w = 0 or
                                  h = 0: the whole frame. The visible set,
                                  samples and pixels are the whole frame's. */
} lv_render_desc;

typedef struct lv_frame_stats
{
    uint32_t n_visible;       /* visible set size */
    uint32_t n_rendered;      /* rendering set size (after ancestor fallback) */
    uint32_t n_available;     /* NodeAvailability::nAvailable */
    uint32_t n_not_available; /* NodeAvailability::nNotAvailable */
    uint32_t n_visited;       /* octree nodes visited by the selection */
    uint32_t max_level;       /* finest level rendered */
    uint32_t samples_per_ray; /* nSamplesPerRay used */
    uint32_t n_uploaded;      /* bricks streamed into the pool */
    uint64_t n_samples;       /* composited samples */
    uint64_t bytes_uploaded;  /* host->device brick bytes */
    uint32_t n_launches;      /* kernels this library launched for the frame */
    float select_ms;          /* device time of the LOD selection */
    float raycast_ms;         /* device time of the ray-cast kernel */
    uint32_t error_flags;     /* 0, or the device's index-check code: 1 rendering
                                 set overflow, 2 node outside the octree,
                                 3 brick outside the pool (the access was skipped),
                                 4 the selection's grid barrier gave up */
    uint32_t n_passes;        /* 1, or the passes of a frame whose visible set
                                 exceeded the brick pool (renderSync,
                                 RenderPipeline.cpp:92-158) */
    float stream_ms;          /* host time spent fetching and streaming bricks */
} lv_frame_stats;

/* One frame of one view: LOD selection, brick residency (streaming misses
 * from the volume's source into the pool), and the ray cast into d_rgba
 * (width*height float RGBA, row 0 at the bottom, premultiplied colour as the
 * reference's RGBA32F render texture holds it). Replaces
 * RenderPipeline::render (livre/lib/pipeline/RenderPipeline.cpp:268-278) with
 * Renderer::render (livre/core/render/Renderer.cpp:33-47) and the
 * RayCastRenderer shaders. Returns once the frame is enqueued on `stream`:
 * the writes to d_rgba are ordered on `stream` after the caller's earlier
 * work there. The selection, which reads and writes only the context's own
 * buffers, runs on an internal stream; when the previous frame is still in
 * flight it may start before the caller's work queued since that frame. */
lv_status lv_render(lv_ctx* ctx, lv_volume* vol, lv_tf* tf,
                    const lv_render_desc* desc, float* d_rgba, void* stream);

/* Launch shape of lv_render's ray cast; every kind gives the same image.
 *  LV_LAUNCH_GRID: one thread per pixel in tile_w x tile_h blocks (32 to
 *    256 threads, a multiple of 32).
 *  LV_LAUNCH_TILE_QUEUE: a resident grid of tile_w x tile_h-thread CTAs
 *    taking pixel tiles from a device queue.
 *  LV_LAUNCH_WARP_REFILL: a resident grid whose warps take tile_w x tile_h
 *    pixel tiles (32 to 1024 pixels) and hand a lane whose ray has finished
 *    the tile's next pixel every samples_per_check samples (1..64).
 * order (queue kinds): LV_ORDER_RASTER takes tiles row by row;
 * LV_ORDER_LONGEST_FIRST first estimates each tile's cost by the length of
 * its centre ray inside the volume and starts the longest tiles first, so
 * the frame does not end waiting on a few long rays started late.
 * lookahead (all kinds but warp refill): 1 loads the voxels of a ray's next
 * sample before compositing the current one (shorter latency per ray, more
 * registers per thread); 0 does not.
 * Default: {LV_LAUNCH_TILE_GRID, 8, 8, 0, LV_ORDER_LONGEST_FIRST, 1}, the
 * fastest on a 2048^3 volume at 1920x1080: 0.234 ms of ray cast per frame
 * (every brick resident, no L2 flush), against 0.239 ms for 8 x 16 tiles,
 * 0.31 ms without look-ahead, 0.28 ms in raster order, 0.35 ms for warp
 * tiles and 0.37 ms for the persistent tile queue; and the friendliest to
 * other work on the device (no resident grid).
 * No reference counterpart (the reference rasterises one brick at a time,
 * RayCastRenderer.cpp:503-571). */
enum
{
    LV_LAUNCH_GRID = 0,
    LV_LAUNCH_TILE_QUEUE = 1,
    LV_LAUNCH_WARP_REFILL = 2,
    LV_LAUNCH_TILE_GRID = 3, /* one tile_w x tile_h-thread CTA per tile, block i
                                taking the i-th tile of the order: no resident
                                grid, so CTAs retire tile by tile and other
                                kernels (the next frame's selection) interleave */
    LV_LAUNCH_WARP_TILES = 4 /* a resident grid whose warps each take
                                tile_w x tile_h = 32-pixel tiles from the queue
                                on their own (no CTA-wide wait for the slowest
                                warp of a tile) */
};
enum
{
    LV_ORDER_RASTER = 0,
    LV_ORDER_LONGEST_FIRST = 1
};
typedef struct lv_render_launch
{
    uint32_t kind;
    uint32_t tile_w, tile_h;
    uint32_t samples_per_check;
    uint32_t order;
    uint32_t lookahead;
} lv_render_launch;
lv_status lv_set_render_launch(lv_ctx* ctx, const lv_render_launch* cfg);
lv_status lv_get_render_launch(lv_ctx* ctx, lv_render_launch* cfg);

/* Running totals of lv_render on a context since its creation, kept on the
 * host: reading them does not wait for the device (lv_last_stats does). A
 * frame counts once lv_render has returned LV_OK; its bricks and bytes are
 * the ones it streamed before its ray cast; launches as lv_frame_stats. */
typedef struct lv_ctx_totals
{
    uint64_t frames;
    uint64_t bricks_uploaded;
    uint64_t bytes_uploaded;
    uint64_t launches;
} lv_ctx_totals;
lv_status lv_get_totals(lv_ctx* ctx, lv_ctx_totals* out);

/* The histogram a view's frame feeds the transfer-function editor
 * (HistogramFilter::execute, livre/lib/pipeline/HistogramFilter.cpp:77-149):
 * lv_histogram of the bricks of the last lv_render frame whose world-box
 * centre projects into the rect it rendered (the frame's borders pushed out
 * to infinity, edges half-open), so the histograms of the sort-first tiles
 * of a frame add up to the whole frame's. Waits for the frame. */
lv_status lv_frame_histogram(lv_ctx* ctx, uint32_t n_bins, float range_lo, float range_hi,
                             uint64_t* accumulated);

/* Statistics of the last lv_render / lv_render_batch call (synchronises with
 * its stream). */
lv_status lv_last_stats(lv_ctx* ctx, lv_frame_stats* out);

/* --------------------------------------------------------- batched mode */

typedef struct lv_batch lv_batch;

/* One view of a batch. desc.synchronous is ignored: a batch renders the
 * nearest resident ancestor of a missing brick and streams up to
 * desc.max_uploads misses per view before the next launch (the reference's
 * asynchronous mode, livre/lib/pipeline/RenderPipeline.cpp:160-225).
 * desc.lod.range must be {0, 1}. */
typedef struct lv_batch_view
{
    lv_volume* volume;
    lv_tf* tf;
    lv_render_desc desc;
    float* d_rgba; /* width*height RGBA32F on the device */
} lv_batch_view;

/* Work queues of the persistent ray-cast kernels. */
enum
{
    LV_QUEUE_CTA_TILES = 0,  /* a CTA per work item: tile_w x tile_h threads,
                                one ray each */
    LV_QUEUE_WARP_REFILL = 1, /* a warp per work item: the tile's pixels are
                                 handed to lanes as their rays finish */
    LV_QUEUE_VIEW_KERNELS = 2 /* one ray cast per view (lv_render's one-CTA-per-
                                 tile kernel, view constants as kernel
                                 parameters) on parallel streams, so a view's
                                 last tiles overlap the next view. With
                                 use_graph the whole batch is captured on
                                 every call and applied to the cached
                                 executable graph (cudaGraphExecUpdate): one
                                 graph launch per batch. The default. */
};

/* Launch shape of the persistent ray-cast kernel. */
typedef struct lv_batch_config
{
    uint32_t tile_w, tile_h; /* pixels per work item; CTA tiles: = threads per
                                CTA (a multiple of 32, at most 256); warp
                                refill: 32 to 1024 pixels */
    uint32_t ctas_per_sm;    /* persistent grid = SMs * ctas_per_sm; 0 = as
                                many CTAs as are resident at once */
    uint32_t tf_shared;      /* 1: transfer function staged in shared memory
                                (CTA tiles only) */
    uint32_t use_graph;      /* 1: replay the batch as one CUDA graph */
    uint32_t queue;          /* LV_QUEUE_* */
    uint32_t samples_per_check; /* warp refill: samples a lane takes between
                                   refills (1..64) */
    uint32_t order;          /* LV_ORDER_* (CTA tiles): longest first ranks the
                                (view, tile) items of all views by the
                                estimated samples of their centre ray */
    uint32_t lookahead;      /* view kernels: 1 = one-sample look-ahead (the
                                voxels of the next sample load while the
                                current one composites), as lv_render_launch.
                                The default configuration is lv_render's
                                launch: view kernels, 8 x 8 tiles, longest
                                first, look-ahead 1 */
} lv_batch_config;

/* A batch renderer on ctx (its own stream, graphs and per-view buffers).
 * No reference counterpart: Livre renders one view per channel. */
lv_status lv_batch_create(lv_ctx* ctx, lv_batch** out);
void lv_batch_destroy(lv_batch* batch);
lv_status lv_batch_set_config(lv_batch* batch, const lv_batch_config* cfg);
lv_status lv_batch_get_config(const lv_batch* batch, lv_batch_config* cfg);
/* Renders n views: one multi-view LOD selection, one residency pass and
 * one persistent ray-cast launch per voxel type, fed by a device work queue
 * of (view, tile) items and replayed as a CUDA graph. Ordered after the work
 * already queued on `stream`; `stream` waits for the batch. */
lv_status lv_batch_render(lv_batch* batch, const lv_batch_view* views,
                          uint32_t n, void* stream);
/* Per-view statistics of the last lv_batch_render (synchronises with it);
 * batch_ms / raycast_ms (nullable) receive the device time of the whole
 * batch (CUDA events around it) and of the persistent ray-cast launches
 * (device global timer, first CTA start to last CTA end). */
lv_status lv_batch_stats(lv_batch* batch, lv_frame_stats* out, uint32_t n,
                         float* batch_ms, float* raycast_ms);
/* CUDA-graph cache of a batch: graphs instantiated (`captures`) and
 * launches of an already instantiated graph (`replays`) so far, and the
 * graphs held now. Persistent queues: a batch of n views runs as a launch
 * for the next power of two (padded with empty views), so batch sizes 1..64
 * share 7 graphs per set of kernel variants, replayed as captured. Per-view
 * kernels: every call is captured and, when its graph has the cached one's
 * topology, applied to it by an update and counted as a replay. */
lv_status lv_batch_graph_stats(lv_batch* batch, uint64_t* captures,
                               uint64_t* replays, uint32_t* cached);
/* Times the persistent ray cast on this batch (reps timed launches each)
 * for CTA tiles of {8x8, 16x8, 8x16, 16x16, 32x4, 32x8} pixels with and
 * without transfer-function staging in raster and longest-first order, per-view
 * kernels of {8x8, 8x16} tiles in both orders, and for warp-refill tiles of {8x4, 8x8,
 * 16x8, 16x16} pixels with refills every {2, 8, 32} samples, all on a
 * resident grid; keeps the fastest configuration and returns it in
 * `chosen`. */
lv_status lv_batch_autotune(lv_batch* batch, const lv_batch_view* views,
                            uint32_t n, void* stream, uint32_t reps,
                            lv_batch_config* chosen);
/* Every configuration the last lv_batch_autotune of this batch ran, with its
 * mean ray-cast time in ms (up to `capacity`; *n = how many it ran). */
lv_status lv_batch_autotune_results(const lv_batch* batch, lv_batch_config* configs,
                                    float* raycast_ms, uint32_t capacity, uint32_t* n);

/* -------------------------------------------------------------- serving */

typedef struct lv_server lv_server;

enum
{
    LV_SERVE_BATCHED = 0, /* continuous batching through lv_batch_render */
    LV_SERVE_PLAIN = 1    /* one lv_render per request, in arrival order */
};

typedef struct lv_server_config
{
    uint32_t mode;        /* LV_SERVE_BATCHED or LV_SERVE_PLAIN */
    uint32_t max_batch;   /* requests per launch */
    uint32_t max_queue;   /* submit returns LV_EAGAIN beyond this (0 = no limit) */
    uint32_t use_graph;   /* replay batches as CUDA graphs */
    uint32_t tile_w, tile_h, ctas_per_sm; /* 0 = batch defaults */
    uint64_t max_pixels;  /* pixels per launch, 0 = no limit (a request larger
                             than the budget still runs, alone) */
} lv_server_config;

/* One render request: the output buffer (width*height RGBA32F, device) must
 * stay valid until lv_server_wait returns for it. */
typedef struct lv_request
{
    lv_volume* volume;
    lv_tf* tf;
    lv_render_desc desc;
    float* d_rgba;
} lv_request;

typedef struct lv_request_result
{
    uint32_t status;    /* lv_status of the request */
    uint32_t batch_size;/* requests rendered in the same launch */
    double latency_ms;  /* submit -> frame complete on the device */
    double queue_ms;    /* submit -> admitted (bricks resident, pinned) */
    lv_frame_stats stats;
} lv_request_result;

/* A render server on ctx with its own thread. Requests are admitted in
 * arrival order while the brick pool can hold their missing bricks (free
 * slots plus resident bricks that no admitted request uses), their visible
 * bricks are pinned until they complete, and admitted requests are rendered
 * together while the next ones are admitted (continuous batching). Create the
 * volumes first. No reference counterpart (Livre renders one view per
 * Equalizer channel). */
lv_status lv_server_create(lv_ctx* ctx, const lv_server_config* cfg,
                           lv_server** out);
/* Queues a request (any thread); `ticket` identifies it for lv_server_wait. */
lv_status lv_server_submit(lv_server* server, const lv_request* req,
                           uint64_t* ticket);
/* Waits up to timeout_ms for a request; LV_ETIMEDOUT if it is not done. On
 * LV_OK the result is returned and the ticket is released. */
lv_status lv_server_wait(lv_server* server, uint64_t ticket,
                         uint32_t timeout_ms, lv_request_result* out);
lv_status lv_server_counters(lv_server* server, uint64_t* completed,
                             uint64_t* batches, uint64_t* queued);
/* Where the server thread's time went, summed since creation (batched
 * mode; the plain mode reports its lv_render calls as launch_ms and their
 * device time as device_ms). */
typedef struct lv_server_profile
{
    uint64_t batches, requests, graph_captures;
    double select_ms;  /* admission selections: host wall time */
    double stream_ms;  /* streaming admitted misses: host wall time */
    double launch_ms;  /* enqueuing batches (graph capture included) */
    double wait_ms;    /* blocked on in-flight batches */
    double device_ms;  /* device time of the batches (events around each) */
    double raycast_ms; /* of which the ray-cast launches */
    double select_device_ms; /* admission selections: device time of their
                                kernels (events around them) */
    double select_ids_ms;    /* admission selections: host wall time from
                                their kernels' end to the visible ids on the
                                host */
} lv_server_profile;
lv_status lv_server_get_profile(lv_server* server, lv_server_profile* out);
/* Finishes every queued request, then stops the server thread. */
void lv_server_destroy(lv_server* server);

/* RGBA32F -> RGBA8 (alpha forced to 255 like the framebuffer copy of
 * livre/eq/render/shaders/fragTexCopy.glsl:11-15 onto the RGB window of
 * livre/eq/Window.cpp:122-124), truncating x * 255 after clamping to [0,1]. */
lv_status lv_frame_to_rgba8(lv_ctx* ctx, const float* d_rgba, uint32_t width,
                            uint32_t height, uint8_t* d_out, void* stream);

/* The frame grab (livre/eq/FrameGrabber.cpp:55-111 encodes the channel image
 * as JPEG): an RGBA8 frame (host, row 0 at the bottom) as a lossless PNG
 * written top row first. out = NULL returns the size only; LV_ENOMEM when
 * capacity is too small. No context or device needed. */
lv_status lv_frame_encode_png(const uint8_t* rgba8, uint32_t width, uint32_t height,
                              uint8_t* out, size_t capacity, size_t* size);
/* An RGBA32F device frame converted like lv_frame_to_rgba8 and written to
 * `path` as PNG. Synchronous: waits for the device (work queued on any
 * stream, such as the frame's own ray cast) first. */
lv_status lv_frame_write_png(lv_ctx* ctx, const float* d_rgba, uint32_t width,
                             uint32_t height, const char* path);

#ifdef __cplusplus
}
#endif
#endif
