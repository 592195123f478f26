"""ctypes declarations of the C ABI in include/livre_gb300.h.

The shared library is built in-tree by livre_gb300/build.py. Loading never
falls back to anything else: if the library is missing or fails to load,
``lib()`` raises.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "liblivre_gb300.so")

LV_OK, LV_EINVAL, LV_ENOMEM, LV_ETIMEDOUT, LV_EDEVICE, LV_ENOTFOUND, LV_EAGAIN = range(7)
STATUS_NAMES = {0: "LV_OK", 1: "LV_EINVAL", 2: "LV_ENOMEM", 3: "LV_ETIMEDOUT",
                4: "LV_EDEVICE", 5: "LV_ENOTFOUND", 6: "LV_EAGAIN"}

DT_FLOAT, DT_UINT8, DT_UINT16, DT_UINT32, DT_INT8, DT_INT16, DT_INT32 = range(7)
FILTER_NEAREST, FILTER_TRILINEAR = 0, 1
STEP_REFERENCE, STEP_HALF_VOXEL = 0, 1
BLOB_DEVICE, BLOB_HOST = 0, 1
FBM_DEVICE, FBM_HOST = 0, 1
SEL_WRITTEN, SEL_FOUND, SEL_VISITED, SEL_MAX_LEVEL, SEL_OVERFLOW = range(5)
SELECT_RESULT_WORDS = 8


class VolumeInfo(C.Structure):
    _fields_ = [("voxels", C.c_uint32 * 3), ("max_block", C.c_uint32 * 3),
                ("overlap", C.c_uint32 * 3), ("dtype", C.c_uint32),
                ("comp_count", C.c_uint32), ("world_space_per_voxel", C.c_float),
                ("world_size", C.c_float * 3), ("depth", C.c_uint32),
                ("root_blocks", C.c_uint32 * 3)]


class Camera(C.Structure):
    _fields_ = [("modelview", C.c_float * 16), ("projection", C.c_float * 16)]


class LodParams(C.Structure):
    _fields_ = [("window_height", C.c_uint32), ("screen_space_error", C.c_float),
                ("min_lod", C.c_uint32), ("max_lod", C.c_uint32),
                ("range", C.c_float * 2), ("time_step", C.c_uint32),
                ("n_clip_planes", C.c_uint32), ("clip_planes", (C.c_float * 4) * 6)]


class BlobDesc(C.Structure):
    _fields_ = [("n_blobs", C.c_uint32), ("noise", C.c_uint32), ("seed", C.c_uint64)]


class FbmParams(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("octaves", C.c_uint32), ("lacunarity", C.c_float),
                ("gain", C.c_float), ("frequency", C.c_float)]


class RenderDesc(C.Structure):
    _fields_ = [("camera", Camera), ("width", C.c_uint32), ("height", C.c_uint32),
                ("lod", LodParams), ("samples_per_ray", C.c_uint32),
                ("step_policy", C.c_uint32), ("early_exit", C.c_float),
                ("filter", C.c_uint32), ("data_range", C.c_float * 2),
                ("synchronous", C.c_uint32), ("max_uploads", C.c_uint32),
                ("rect", C.c_uint32 * 4)]


class FrameStats(C.Structure):
    _fields_ = [("n_visible", C.c_uint32), ("n_rendered", C.c_uint32),
                ("n_available", C.c_uint32), ("n_not_available", C.c_uint32),
                ("n_visited", C.c_uint32), ("max_level", C.c_uint32),
                ("samples_per_ray", C.c_uint32), ("n_uploaded", C.c_uint32),
                ("n_samples", C.c_uint64), ("bytes_uploaded", C.c_uint64),
                ("n_launches", C.c_uint32), ("select_ms", C.c_float),
                ("raycast_ms", C.c_float), ("error_flags", C.c_uint32),
                ("n_passes", C.c_uint32), ("stream_ms", C.c_float)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class CtxTotals(C.Structure):
    _fields_ = [("frames", C.c_uint64), ("bricks_uploaded", C.c_uint64),
                ("bytes_uploaded", C.c_uint64), ("launches", C.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchView(C.Structure):
    _fields_ = [("volume", C.c_void_p), ("tf", C.c_void_p), ("desc", RenderDesc),
                ("d_rgba", C.c_void_p)]


BRICKS_QUADS = 0
BRICKS_COMPACT = 1

QUEUE_CTA_TILES = 0
QUEUE_WARP_REFILL = 1
QUEUE_VIEW_KERNELS = 2


class BatchConfig(C.Structure):
    _fields_ = [("tile_w", C.c_uint32), ("tile_h", C.c_uint32), ("ctas_per_sm", C.c_uint32),
                ("tf_shared", C.c_uint32), ("use_graph", C.c_uint32), ("queue", C.c_uint32),
                ("samples_per_check", C.c_uint32), ("order", C.c_uint32),
                ("lookahead", C.c_uint32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


LAUNCH_GRID = 0
LAUNCH_TILE_QUEUE = 1
LAUNCH_WARP_REFILL = 2
LAUNCH_TILE_GRID = 3
LAUNCH_WARP_TILES = 4
ORDER_RASTER = 0
ORDER_LONGEST_FIRST = 1


class RenderLaunch(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("tile_w", C.c_uint32), ("tile_h", C.c_uint32),
                ("samples_per_check", C.c_uint32), ("order", C.c_uint32),
                ("lookahead", C.c_uint32)]


class ServerProfile(C.Structure):
    _fields_ = [("batches", C.c_uint64), ("requests", C.c_uint64),
                ("graph_captures", C.c_uint64), ("select_ms", C.c_double),
                ("stream_ms", C.c_double), ("launch_ms", C.c_double),
                ("wait_ms", C.c_double), ("device_ms", C.c_double),
                ("raycast_ms", C.c_double), ("select_device_ms", C.c_double),
                ("select_ids_ms", C.c_double)]


class ServerConfig(C.Structure):
    _fields_ = [("mode", C.c_uint32), ("max_batch", C.c_uint32), ("max_queue", C.c_uint32),
                ("use_graph", C.c_uint32), ("tile_w", C.c_uint32), ("tile_h", C.c_uint32),
                ("ctas_per_sm", C.c_uint32), ("max_pixels", C.c_uint64)]


class Request(C.Structure):
    _fields_ = [("volume", C.c_void_p), ("tf", C.c_void_p), ("desc", RenderDesc),
                ("d_rgba", C.c_void_p)]


class RequestResult(C.Structure):
    _fields_ = [("status", C.c_uint32), ("batch_size", C.c_uint32), ("latency_ms", C.c_double),
                ("queue_ms", C.c_double), ("stats", FrameStats)]


SERVE_BATCHED, SERVE_PLAIN = 0, 1

GET_DATA_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint64, C.c_void_p, C.c_size_t)

P = C.POINTER
_SIGNATURES = {
    "lv_fill_regular_volume_info": (C.c_int, [P(VolumeInfo)]),
    "lv_brick_slot_bytes": (C.c_int, [C.c_void_p, P(VolumeInfo), P(C.c_uint64)]),
    "lv_pool_set_brick_layout": (C.c_int, [C.c_void_p, C.c_uint32]),
    "lv_ctx_create": (C.c_int, [C.c_int, P(C.c_void_p)]),
    "lv_ctx_destroy": (None, [C.c_void_p]),
    "lv_last_error": (C.c_char_p, [C.c_void_p]),
    "lv_abi_version": (C.c_uint32, []),
    "lv_select_visible": (C.c_int, [C.c_void_p, P(VolumeInfo), P(Camera), P(LodParams),
                                    C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    "lv_select_visible_noalloc": (C.c_int, [P(VolumeInfo), P(Camera), P(LodParams), C.c_void_p,
                                            C.c_uint32, C.c_void_p, C.c_void_p]),
    "lv_test_fail_grid_barrier": (C.c_int, [C.c_void_p, C.c_uint32]),
    "lv_select_visible_host": (C.c_int, [C.c_void_p, P(VolumeInfo), P(Camera), P(LodParams),
                                         C.c_void_p, C.c_uint32, C.c_void_p]),
    "lv_pool_configure": (C.c_int, [C.c_void_p, C.c_size_t]),
    "lv_pool_purge": (C.c_int, [C.c_void_p]),
    "lv_volume_create": (C.c_int, [C.c_void_p, P(VolumeInfo), GET_DATA_FN, C.c_void_p,
                                   P(C.c_void_p)]),
    "lv_volume_create_blob": (C.c_int, [C.c_void_p, P(VolumeInfo), P(BlobDesc), C.c_uint32,
                                        P(C.c_void_p)]),
    "lv_volume_destroy": (None, [C.c_void_p]),
    "lv_volume_get_info": (C.c_int, [C.c_void_p, P(VolumeInfo)]),
    "lv_volume_open": (C.c_int, [C.c_void_p, C.c_char_p, P(C.c_void_p)]),
    "lv_volume_get_data": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_size_t]),
    "lv_histogram": (C.c_int, [C.c_void_p, P(C.c_uint64), C.c_uint32, C.c_uint32, C.c_float,
                               C.c_float, P(C.c_uint64), P(C.c_uint64)]),
    "lv_volume_load": (C.c_int, [C.c_void_p, P(C.c_uint64), C.c_uint32, P(C.c_uint32)]),
    "lv_volume_resident": (C.c_int, [C.c_void_p, P(C.c_uint64), C.c_uint32, P(C.c_uint32)]),
    "lv_blob_generate": (C.c_int, [C.c_void_p, P(VolumeInfo), P(BlobDesc), P(C.c_uint64),
                                   C.c_uint32, C.c_void_p, C.c_void_p]),
    "lv_frame_encode_png": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p,
                                      C.c_size_t, P(C.c_size_t)]),
    "lv_frame_write_png": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                     C.c_char_p]),
    "lv_volume_create_fbm": (C.c_int, [C.c_void_p, P(VolumeInfo), P(FbmParams), C.c_uint32,
                                       C.c_uint32, P(C.c_void_p)]),
    "lv_fbm_brick": (C.c_int, [P(VolumeInfo), P(FbmParams), C.c_uint64, C.c_void_p,
                               C.c_uint32]),
    "lv_fbm_generate": (C.c_int, [C.c_void_p, P(VolumeInfo), P(FbmParams), P(C.c_uint64),
                                  C.c_uint32, C.c_void_p, C.c_void_p]),
    "lv_tf_create": (C.c_int, [C.c_void_p, P(C.c_float), C.c_uint32, P(C.c_void_p)]),
    "lv_tf_destroy": (None, [C.c_void_p]),
    "lv_render": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, P(RenderDesc), C.c_void_p,
                            C.c_void_p]),
    "lv_last_stats": (C.c_int, [C.c_void_p, P(FrameStats)]),
    "lv_get_totals": (C.c_int, [C.c_void_p, P(CtxTotals)]),
    "lv_frame_histogram": (C.c_int, [C.c_void_p, C.c_uint32, C.c_float, C.c_float,
                                     P(C.c_uint64)]),
    "lv_batch_create": (C.c_int, [C.c_void_p, P(C.c_void_p)]),
    "lv_batch_destroy": (None, [C.c_void_p]),
    "lv_batch_set_config": (C.c_int, [C.c_void_p, P(BatchConfig)]),
    "lv_batch_get_config": (C.c_int, [C.c_void_p, P(BatchConfig)]),
    "lv_batch_render": (C.c_int, [C.c_void_p, P(BatchView), C.c_uint32, C.c_void_p]),
    "lv_batch_stats": (C.c_int, [C.c_void_p, P(FrameStats), C.c_uint32, P(C.c_float),
                                 P(C.c_float)]),
    "lv_batch_autotune": (C.c_int, [C.c_void_p, P(BatchView), C.c_uint32, C.c_void_p,
                                    C.c_uint32, P(BatchConfig)]),
    "lv_batch_autotune_results": (C.c_int, [C.c_void_p, P(BatchConfig), P(C.c_float),
                                            C.c_uint32, P(C.c_uint32)]),
    "lv_server_create": (C.c_int, [C.c_void_p, P(ServerConfig), P(C.c_void_p)]),
    "lv_server_submit": (C.c_int, [C.c_void_p, P(Request), P(C.c_uint64)]),
    "lv_server_wait": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint32, P(RequestResult)]),
    "lv_set_render_launch": (C.c_int, [C.c_void_p, P(RenderLaunch)]),
    "lv_get_render_launch": (C.c_int, [C.c_void_p, P(RenderLaunch)]),
    "lv_server_get_profile": (C.c_int, [C.c_void_p, P(ServerProfile)]),
    "lv_batch_graph_stats": (C.c_int, [C.c_void_p, P(C.c_uint64), P(C.c_uint64),
                                       P(C.c_uint32)]),
    "lv_server_counters": (C.c_int, [C.c_void_p, P(C.c_uint64), P(C.c_uint64),
                                     P(C.c_uint64)]),
    "lv_server_destroy": (None, [C.c_void_p]),
    "lv_frame_to_rgba8": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                    C.c_void_p, C.c_void_p]),
    "lv_register_source": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p]),
    "lv_source_descriptions": (C.c_int, [C.c_void_p, C.c_size_t, P(C.c_size_t)]),
    "lv_unregister_source": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lv_source_probe": (C.c_int, [C.c_char_p, P(VolumeInfo)]),
    "lv_volume_set_fetch_threads": (C.c_int, [C.c_void_p, C.c_uint32]),
    "lv_volume_get_fetch_threads": (C.c_int, [C.c_void_p, P(C.c_uint32)]),
    "lv_source_open": (C.c_int, [C.c_char_p, P(VolumeInfo), P(C.c_void_p), P(C.c_void_p),
                                 P(C.c_void_p)]),
    "lv_load_plugins": (C.c_int, [C.c_char_p, C.c_char_p, P(C.c_uint32)]),
    "lv_source_handles": (C.c_int, [C.c_char_p]),
}

_lib = None


def lib():
    """Loads liblivre_gb300.so (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("livre_gb300 native library not built: %s "
                               "(run __graft_entry__.build() or livre_gb300/build.py)" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class LivreError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))
        self.status = status


def check(status, ctx=None):
    if status != LV_OK:
        msg = lib().lv_last_error(ctx).decode() if ctx else ""
        raise LivreError(status, msg)
