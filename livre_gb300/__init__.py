"""livre_gb300: GB300-native rendering hot path of BlueBrain/Livre.

Python mirror of the reference's interfaces for this path, over the C ABI of
include/livre_gb300.h (liblivre_gb300.so, built in-tree):

  NodeId                   livre/data/NodeId.h:31-160
  VolumeInformation        livre/data/VolumeInformation.h:42-111
  fill_regular_volume_info livre/data/DataSourcePlugin.cpp:73-95
  VolumeRendererParameters livre/lib/zeroeq/volumeRendererParameters.fbs:4-14
  TransferFunction1D       livre/core/render/TransferFunction1D.cpp:28-107
  Context.select_visible   DFSTraversal + SelectVisibles
  Context.render           RenderPipeline::render + RayCastRenderer

Device buffers are torch CUDA tensors; torch is only the allocator and
stream provider. Every computation runs in the native library.
"""
import atexit
import ctypes as C
import dataclasses
import math
import sys
import weakref

import numpy as np

from . import _abi
from ._abi import (BLOB_DEVICE, BLOB_HOST, BRICKS_COMPACT, BRICKS_QUADS, DT_UINT8, DT_UINT16, FBM_DEVICE, FBM_HOST,
                   FILTER_NEAREST,
                   FILTER_TRILINEAR, LAUNCH_GRID, LAUNCH_TILE_GRID, LAUNCH_TILE_QUEUE,
                   LAUNCH_WARP_REFILL, LAUNCH_WARP_TILES,
                   ORDER_LONGEST_FIRST, ORDER_RASTER,
                   QUEUE_CTA_TILES, QUEUE_VIEW_KERNELS, QUEUE_WARP_REFILL, STEP_HALF_VOXEL,
                   STEP_REFERENCE, LivreError, check, lib)

__all__ = ["NodeId", "VolumeInformation", "VolumeRendererParameters", "TransferFunction1D",
           "Context", "perspective", "look_at", "orbit_camera", "LivreError"]

# ----------------------------------------------------------------- NodeId
LEVEL_BITS, BLOCK_BITS, TIMESTEP_BITS = 4, 14, 18
INVALID_NODE_ID = (1 << 64) - 1
INVALID_LEVEL = (1 << LEVEL_BITS) - 1


class NodeId:
    """64-bit octree node id: level:4, x:14, y:14, z:14, timeStep:18 (NodeId.h:34-49)."""
    __slots__ = ("id",)

    def __init__(self, ident=INVALID_NODE_ID, position=None, time_step=0):
        if position is None:
            self.id = int(ident) & INVALID_NODE_ID
        else:
            level = int(ident)
            x, y, z = (int(p) for p in position)
            self.id = ((level & 0xF) | ((x & 0x3FFF) << 4) | ((y & 0x3FFF) << 18)
                       | ((z & 0x3FFF) << 32) | ((int(time_step) & 0x3FFFF) << 46))

    level = property(lambda s: s.id & 0xF)
    time_step = property(lambda s: s.id >> 46)
    position = property(lambda s: ((s.id >> 4) & 0x3FFF, (s.id >> 18) & 0x3FFF,
                                   (s.id >> 32) & 0x3FFF))

    def is_valid(self):
        return self.level != INVALID_LEVEL

    def is_root(self):
        return self.level == 0

    def get_parent(self):
        """NodeId.cpp:63-70."""
        if self.level in (INVALID_LEVEL, 0):
            return NodeId()
        x, y, z = self.position
        return NodeId(self.level - 1, (x // 2, y // 2, z // 2), self.time_step)

    def get_parents(self):
        out, p = [], self.get_parent()
        while p.is_valid():
            out.append(p)
            p = p.get_parent()
        return out

    def get_children(self):
        """NodeId.cpp:92-114: x outer, y, z inner."""
        if self.level == INVALID_LEVEL:
            return []
        x, y, z = (2 * p for p in self.position)
        return [NodeId(self.level + 1, (x + i, y + j, z + k), self.time_step)
                for i in range(2) for j in range(2) for k in range(2)]

    def is_parent(self, parent):
        """NodeId.cpp:72-86, including the reference's left shift of the
        child position (true only when both positions are 0)."""
        if parent.level >= self.level or parent.time_step != self.time_step or parent.id == self.id:
            return False
        d = self.level - parent.level
        return all((c << d) == p for c, p in zip(self.position, parent.position))

    def __eq__(self, o):
        return self.id == (o.id if isinstance(o, NodeId) else int(o))

    def __hash__(self):
        return hash(self.id)

    def __lt__(self, o):
        return self.id < (o.id if isinstance(o, NodeId) else int(o))

    def __int__(self):
        return self.id

    def __repr__(self):
        return "NodeId(level=%d, position=%s, time_step=%d)" % (self.level, self.position,
                                                                 self.time_step)


# ------------------------------------------------------ VolumeInformation
class VolumeInformation:
    """livre::VolumeInformation for a regular octree volume."""

    def __init__(self, voxels, block, overlap=0, dtype=DT_UINT8):
        self.info = _abi.VolumeInfo()
        vox = voxels if hasattr(voxels, "__len__") else (voxels,) * 3
        blk = block if hasattr(block, "__len__") else (block,) * 3
        ovl = overlap if hasattr(overlap, "__len__") else (overlap,) * 3
        for i in range(3):
            self.info.voxels[i] = int(vox[i])
            self.info.overlap[i] = int(ovl[i])
            self.info.max_block[i] = int(blk[i]) + 2 * int(ovl[i])
        self.info.dtype = dtype
        self.info.comp_count = 1
        fill_regular_volume_info(self)

    depth = property(lambda s: s.info.depth)
    root_blocks = property(lambda s: tuple(s.info.root_blocks))
    world_size = property(lambda s: tuple(s.info.world_size))
    world_space_per_voxel = property(lambda s: s.info.world_space_per_voxel)
    voxels = property(lambda s: tuple(s.info.voxels))
    max_block = property(lambda s: tuple(s.info.max_block))
    overlap = property(lambda s: tuple(s.info.overlap))
    dtype = property(lambda s: s.info.dtype)
    comp_count = property(lambda s: s.info.comp_count)

    @property
    def block_size(self):
        return tuple(m - 2 * o for m, o in zip(self.max_block, self.overlap))

    @property
    def bytes_per_voxel(self):
        return {0: 4, 1: 1, 2: 2, 3: 4, 4: 1, 5: 2, 6: 4}[self.dtype]

    @property
    def brick_bytes(self):
        return int(np.prod(self.max_block)) * self.bytes_per_voxel

    @property
    def slot_bytes(self):
        """Pool bytes one brick occupies in the default brick layout
        (lv_brick_slot_bytes; Context.slot_bytes for a context's layout)."""
        out = C.c_uint64()
        check(lib().lv_brick_slot_bytes(None, C.byref(self.info), C.byref(out)))
        return int(out.value)

    def node_count(self):
        r = self.root_blocks
        return sum((r[0] << l) * (r[1] << l) * (r[2] << l) for l in range(self.depth))

    def all_nodes(self, time_step=0):
        r = self.root_blocks
        for l in range(self.depth):
            for x in range(r[0] << l):
                for y in range(r[1] << l):
                    for z in range(r[2] << l):
                        yield NodeId(l, (x, y, z), time_step)


def fill_regular_volume_info(vol):
    check(lib().lv_fill_regular_volume_info(C.byref(vol.info)))
    return vol


# ------------------------------------------------ VolumeRendererParameters
@dataclasses.dataclass
class VolumeRendererParameters:
    """Defaults of livre/lib/zeroeq/volumeRendererParameters.fbs:4-14."""
    max_lod: int = 9
    min_lod: int = 0
    screen_space_error: float = 4.0
    synchronous_mode: bool = False
    samples_per_ray: int = 0
    max_gpu_cache_memory: int = 3072  # MiB
    max_cpu_cache_memory: int = 8192  # MiB
    show_axes: bool = False
    linear_filtering: bool = False


# ----------------------------------------------------- TransferFunction1D
class TransferFunction1D:
    """RGBA float transfer function (TransferFunction1D.cpp:28-107)."""

    def __init__(self, rgba=None):
        self.rgba = default_transfer_function() if rgba is None else np.ascontiguousarray(
            rgba, np.float32).reshape(-1, 4)

    @classmethod
    def from_file(cls, path):
        """`.1dt` loader; a missing file or another extension yields the default
        (TransferFunction1D.cpp:28-54)."""
        try:
            if not path.endswith(".1dt"):
                raise OSError
            toks = open(path).read().split()
        except OSError:
            return cls()
        n = int(toks[0])
        vals = np.array([float(t) for t in toks[1:1 + 4 * n]], np.float32).reshape(n, 4)
        return cls(vals)

    def get_lut(self):
        """uint8 LUT, truncating x * 255 (TransferFunction1D.cpp:92-107)."""
        return (self.rgba * np.float32(255.0)).astype(np.uint8)


def default_transfer_function():
    """The 256-entry default of TransferFunction1D.cpp:56-90 (FP32)."""
    f = np.float32
    out = np.zeros((256, 4), np.float32)
    c1 = np.array([0, 1, 1], np.float32)
    diff = np.array([1, 0, 1], np.float32) - c1
    a1, a2 = f(0.39), f(0.03)
    d1, d2 = f(127.0), f(255.0)
    for i in range(1, 256):
        fi = f(i)
        if fi <= d1:
            out[i, :3] = c1
            out[i, 3] = a1 * (fi / d1)
        else:
            w = (fi - d1 + f(1.0)) / (d2 - d1 + f(1.0))
            out[i, :3] = w * diff + c1
            out[i, 3] = w * (a2 - a1) + a1
    return out


def linear_ramp_tf(n=256):
    """Every channel of entry i is i / (n - 1)."""
    v = np.arange(n, dtype=np.float32) / np.float32(n - 1)
    return np.repeat(v[:, None], 4, axis=1).astype(np.float32)


def gaussian_peaks_tf(n=256, seed=0, peaks=4):
    """alpha(s) = sum_k h_k exp(-(s - mu_k)^2 / (2 w_k^2)); RGB = weight-blended
    random colour per peak."""
    rng = np.random.default_rng(seed)
    s = (np.arange(n, dtype=np.float64) + 0.5) / n
    mu = rng.uniform(0.15, 0.95, peaks)
    w = rng.uniform(0.02, 0.08, peaks)
    h = rng.uniform(0.2, 0.9, peaks)
    col = rng.uniform(0.1, 1.0, (peaks, 3))
    g = h[None, :] * np.exp(-((s[:, None] - mu[None, :]) ** 2) / (2 * w[None, :] ** 2))
    alpha = np.clip(g.sum(1), 0, 1)
    wt = g / np.maximum(g.sum(1, keepdims=True), 1e-12)
    rgb = wt @ col
    return np.concatenate([rgb, alpha[:, None]], 1).astype(np.float32)


# ------------------------------------------------------------- cameras
def encode_png(rgba8):
    """PNG bytes of an (H, W, 4) uint8 frame whose row 0 is the bottom row."""
    a = np.ascontiguousarray(rgba8, np.uint8)
    H, W = a.shape[:2]
    size = C.c_size_t()
    check(lib().lv_frame_encode_png(a.ctypes.data, W, H, None, 0, C.byref(size)))
    out = (C.c_uint8 * size.value)()
    check(lib().lv_frame_encode_png(a.ctypes.data, W, H, out, size.value, C.byref(size)))
    return bytes(out)


# ------------------------------------------------------------- data-source plugins
def load_plugins(paths=None, pattern=None):
    """DataSource::loadPlugins: loads the plugin libraries matching `pattern`
    (default "Livre.*Source") from the ':'-separated `paths` (default
    LD_LIBRARY_PATH); returns how many were newly loaded."""
    n = C.c_uint32()
    check(lib().lv_load_plugins(None if paths is None else paths.encode(),
                                None if pattern is None else pattern.encode(), C.byref(n)))
    return n.value


def source_handles(uri):
    """DataSource::handles: True when a registered or built-in source opens `uri`."""
    return bool(lib().lv_source_handles(uri.encode()))


def probe_source(uri):
    """The VolumeInformation a registered plugin source gives for `uri`."""
    info = _abi.VolumeInfo()
    check(lib().lv_source_probe(uri.encode(), C.byref(info)))
    vi = VolumeInformation.__new__(VolumeInformation)
    vi.info = info
    return vi


def source_descriptions():
    """DataSource::getDescriptions: registered sources first, then built-in."""
    n = C.c_size_t()
    check(lib().lv_source_descriptions(None, 0, C.byref(n)))
    buf = C.create_string_buffer(n.value)
    check(lib().lv_source_descriptions(buf, n.value, C.byref(n)))
    return buf.value.decode()


class DataSource:
    """livre::DataSource on the host (lv_source_open): the volume description
    and bricks of a URI, read without a context or device."""

    def __init__(self, uri):
        info = _abi.VolumeInfo()
        fn, src, free = C.c_void_p(), C.c_void_p(), C.c_void_p()
        check(lib().lv_source_open(uri.encode(), C.byref(info), C.byref(fn), C.byref(src),
                                   C.byref(free)))
        self._fn = _abi.GET_DATA_FN(fn.value)
        self._free = C.CFUNCTYPE(None, C.c_void_p)(free.value) if free.value else None
        self._src = src.value
        self.info = VolumeInformation.__new__(VolumeInformation)
        self.info.info = info

    def get_data(self, node_id):
        """The brick of `node_id` (brick_bytes uint8), or None when the
        source has no data for it or it lies outside the octree."""
        nid = NodeId(int(node_id)) if not isinstance(node_id, NodeId) else node_id
        r = self.info.root_blocks
        L = nid.level
        if (not nid.is_valid() or L >= self.info.depth or
                any(p >= (b << L) for p, b in zip(nid.position, r))):
            return None
        out = np.zeros(self.info.brick_bytes, np.uint8)
        if self._fn(self._src, int(nid), out.ctypes.data, out.size) != 0:
            return None
        return out

    def close(self):
        if self._free is not None:
            self._free(self._src)
            self._free = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fbm_params(seed, octaves=6, lacunarity=2.0, gain=0.5, frequency=8.0):
    return _abi.FbmParams(seed, octaves, lacunarity, gain, frequency)


def fbm_brick(vol_info, node_id, seed, octaves=6, lacunarity=2.0, gain=0.5, frequency=8.0,
              n_threads=0):
    """One fBm brick generated on the host (lv_fbm_brick): brick_bytes uint8."""
    out = np.zeros(vol_info.brick_bytes, np.uint8)
    p = fbm_params(seed, octaves, lacunarity, gain, frequency)
    check(lib().lv_fbm_brick(C.byref(vol_info.info), C.byref(p), C.c_uint64(int(node_id)),
                             out.ctypes.data, n_threads))
    return out


def perspective(fovy_deg, aspect, near, far):
    """OpenGL perspective projection, column-major flat (16,) float32."""
    f = 1.0 / math.tan(math.radians(fovy_deg) / 2.0)
    m = np.zeros((4, 4), np.float64)
    m[0, 0] = f / aspect
    m[1, 1] = f
    m[2, 2] = (far + near) / (near - far)
    m[2, 3] = 2 * far * near / (near - far)
    m[3, 2] = -1.0
    return m.T.reshape(16).astype(np.float32)


def look_at(eye, center, up=(0.0, 1.0, 0.0)):
    """View matrix (world -> eye), column-major flat (16,) float32."""
    eye, center, up = (np.asarray(v, np.float64) for v in (eye, center, up))
    fwd = center - eye
    fwd /= np.linalg.norm(fwd)
    s = np.cross(fwd, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, fwd)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -fwd
    m[:3, 3] = -m[:3, :3] @ eye
    return m.T.reshape(16).astype(np.float32)


def orbit_camera(k, n_frames, world_size=(1.0, 1.0, 1.0), width=512, height=512,
                 fovy=45.0, near=0.1, far=15.0, radius_scale=2.5, elevation=0.35):
    """Frame k of an n-frame orbit about +y at 2.5x the volume diagonal."""
    r = radius_scale * float(np.linalg.norm(world_size))
    a = 2.0 * math.pi * k / n_frames
    eye = (r * math.sin(a) * math.cos(elevation), r * math.sin(elevation),
           r * math.cos(a) * math.cos(elevation))
    return look_at(eye, (0, 0, 0)), perspective(fovy, width / height, near, far)


# ------------------------------------------------------------- context
def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


def _stream(stream):
    if stream is None:
        import torch
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return C.c_void_p(stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream))


def make_camera(mv, proj):
    cam = _abi.Camera()
    for i, v in enumerate(np.asarray(mv, np.float32).reshape(16)):
        cam.modelview[i] = float(v)
    for i, v in enumerate(np.asarray(proj, np.float32).reshape(16)):
        cam.projection[i] = float(v)
    return cam


def make_lod(window_height, sse, min_lod=0, max_lod=100, rng=(0.0, 1.0), time_step=0,
             clip_planes=None):
    p = _abi.LodParams()
    p.window_height, p.screen_space_error = window_height, sse
    p.min_lod, p.max_lod = min_lod, max_lod
    p.range[0], p.range[1] = rng
    p.time_step = time_step
    if clip_planes is not None:
        p.n_clip_planes = len(clip_planes)
        for i, pl in enumerate(clip_planes):
            for j in range(4):
                p.clip_planes[i][j] = float(pl[j])
    return p


class Volume:
    def __init__(self, ctx, handle, info, keepalive=None):
        self.ctx, self.handle, self.info, self._keep = ctx, handle, info, keepalive
        ctx._children.add(self)

    def load(self, node_ids):
        """Cache::load of explicit bricks; returns how many were streamed."""
        ids = np.ascontiguousarray([int(i) for i in node_ids], np.uint64)
        n = C.c_uint32()
        check(lib().lv_volume_load(self.handle, ids.ctypes.data_as(C.POINTER(C.c_uint64)),
                                   len(ids), C.byref(n)), self.ctx.handle)
        return n.value

    def get_data(self, node_id):
        """DataSource::getData: the brick's bytes (numpy uint8) or None."""
        out = np.zeros(self.info.brick_bytes, np.uint8)
        st = lib().lv_volume_get_data(self.handle, C.c_uint64(int(node_id)),
                                      out.ctypes.data, out.nbytes)
        if st == _abi.LV_ENOTFOUND:
            return None
        check(st, self.ctx.handle)
        return out

    def histogram(self, node_ids, n_bins=256, data_range=(0.0, 255.0), per_brick=False):
        """Accumulated (and optionally per-brick) value histograms of bricks."""
        ids = np.ascontiguousarray([int(i) for i in node_ids], np.uint64)
        acc = np.zeros(n_bins, np.uint64)
        pb = np.zeros((len(ids), n_bins), np.uint64) if per_brick else None
        check(lib().lv_histogram(self.handle, ids.ctypes.data_as(C.POINTER(C.c_uint64)),
                                 len(ids), n_bins, float(data_range[0]), float(data_range[1]),
                                 pb.ctypes.data_as(C.POINTER(C.c_uint64)) if per_brick else None,
                                 acc.ctypes.data_as(C.POINTER(C.c_uint64))), self.ctx.handle)
        return (acc, pb) if per_brick else acc

    @property
    def fetch_threads(self):
        """Host threads calling the source's getData at once (callback sources)."""
        n = C.c_uint32()
        check(lib().lv_volume_get_fetch_threads(self.handle, C.byref(n)), self.ctx.handle)
        return n.value

    @fetch_threads.setter
    def fetch_threads(self, n):
        check(lib().lv_volume_set_fetch_threads(self.handle, int(n)), self.ctx.handle)

    def resident(self):
        """Resident node ids, oldest load first."""
        n = C.c_uint32()
        cap = max(1, self.info.node_count())
        out = np.zeros(cap, np.uint64)
        check(lib().lv_volume_resident(self.handle, out.ctypes.data_as(C.POINTER(C.c_uint64)),
                                       cap, C.byref(n)), self.ctx.handle)
        return [int(x) for x in out[: n.value]]

    def close(self):
        if self.handle:
            lib().lv_volume_destroy(self.handle)
            self.handle = None
            self.ctx._children.discard(self)

    def __del__(self):
        if sys.is_finalizing():
            return  # CUDA may already be torn down; the OS reclaims everything
        try:
            self.close()
        except Exception:
            pass


class TransferFunction:
    def __init__(self, ctx, rgba):
        self.ctx = ctx
        self.rgba = np.ascontiguousarray(rgba, np.float32).reshape(-1, 4)
        h = C.c_void_p()
        check(lib().lv_tf_create(ctx.handle, self.rgba.ctypes.data_as(C.POINTER(C.c_float)),
                                 self.rgba.shape[0], C.byref(h)), ctx.handle)
        self.handle = h
        ctx._children.add(self)

    def close(self):
        if self.handle:
            lib().lv_tf_destroy(self.handle)
            self.handle = None
            self.ctx._children.discard(self)

    def __del__(self):
        if sys.is_finalizing():
            return  # CUDA may already be torn down; the OS reclaims everything
        try:
            self.close()
        except Exception:
            pass


_live_contexts = weakref.WeakSet()


@atexit.register
def _close_live_contexts():
    """Destroys contexts still open at exit while the CUDA runtime is alive."""
    for ctx in list(_live_contexts):
        try:
            ctx.close()
        except Exception:
            pass


class Context:
    """One CUDA device; owns the brick pool (lv_ctx)."""

    def __init__(self, device=0, pool_bytes=None, brick_layout=None):
        """brick_layout: BRICKS_QUADS (the default) or BRICKS_COMPACT
        (lv_pool_set_brick_layout)."""
        self._children = weakref.WeakSet()
        _live_contexts.add(self)
        self.handle = None
        h = C.c_void_p()
        check(lib().lv_ctx_create(int(device), C.byref(h)))
        self.handle = h
        self.device = device
        if pool_bytes is not None:
            check(lib().lv_pool_configure(h, int(pool_bytes)), h)
        if brick_layout is not None:
            check(lib().lv_pool_set_brick_layout(h, int(brick_layout)), h)

    def slot_bytes(self, vi):
        """Pool bytes one brick of volume description vi occupies on this
        context (lv_brick_slot_bytes)."""
        out = C.c_uint64()
        check(lib().lv_brick_slot_bytes(self.handle, C.byref(vi.info), C.byref(out)),
              self.handle)
        return int(out.value)

    def close(self):
        """Destroys the volumes and transfer functions of this context, then it
        (the C ABI requires children to go first)."""
        if self.handle:
            for child in list(self._children):
                child.close()
            lib().lv_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        if sys.is_finalizing():
            return  # CUDA may already be torn down; the OS reclaims everything
        try:
            self.close()
        except Exception:
            pass

    # -- selection
    def select_visible(self, vol_info, mv, proj, window_height, sse, min_lod=0, max_lod=100,
                       rng=(0.0, 1.0), time_step=0, clip_planes=None, out=None, result=None,
                       stream=None, sync=True):
        """Visible NodeIds (uint64 numpy array, unordered) of one view."""
        import torch
        dev = torch.device("cuda", self.device)
        cap = vol_info.node_count()
        if out is None:
            out = torch.empty(max(cap, 1), dtype=torch.int64, device=dev)
        if result is None:
            result = torch.zeros(_abi.SELECT_RESULT_WORDS, dtype=torch.int32, device=dev)
        cam = make_camera(mv, proj)
        lod = make_lod(window_height, sse, min_lod, max_lod, rng, time_step, clip_planes)
        check(lib().lv_select_visible(self.handle, C.byref(vol_info.info), C.byref(cam),
                                      C.byref(lod), _ptr(out), out.numel(), _ptr(result),
                                      _stream(stream)), self.handle)
        if not sync:
            return out, result
        res = result.cpu().numpy().view(np.uint32)
        n = int(res[_abi.SEL_WRITTEN])
        return out[:n].cpu().numpy().view(np.uint64).copy(), res.copy()

    # -- volumes
    def blob_volume(self, vol_info, n_blobs, seed, noise=0, placement=BLOB_DEVICE):
        d = _abi.BlobDesc(n_blobs, noise, seed)
        h = C.c_void_p()
        check(lib().lv_volume_create_blob(self.handle, C.byref(vol_info.info), C.byref(d),
                                          placement, C.byref(h)), self.handle)
        return Volume(self, h, vol_info)

    def fbm_volume(self, vol_info, seed, octaves=6, lacunarity=2.0, gain=0.5, frequency=8.0,
                   placement=FBM_DEVICE, host_threads=0):
        """Procedural fBm volume (improved Perlin noise), generated per brick on
        the device (FBM_DEVICE) or on the host when it misses (FBM_HOST)."""
        p = fbm_params(seed, octaves, lacunarity, gain, frequency)
        h = C.c_void_p()
        check(lib().lv_volume_create_fbm(self.handle, C.byref(vol_info.info), C.byref(p),
                                         placement, host_threads, C.byref(h)), self.handle)
        return Volume(self, h, vol_info)

    def fbm_bricks(self, vol_info, node_ids, seed, octaves=6, lacunarity=2.0, gain=0.5,
                   frequency=8.0, stream=None):
        """fBm bricks of `node_ids` generated on the device, as a device tensor
        (n, brick_bytes) uint8."""
        import torch
        ids = np.ascontiguousarray(node_ids, np.uint64)
        out = torch.empty((len(ids), vol_info.brick_bytes), dtype=torch.uint8,
                          device=torch.device("cuda", self.device))
        p = fbm_params(seed, octaves, lacunarity, gain, frequency)
        check(lib().lv_fbm_generate(self.handle, C.byref(vol_info.info), C.byref(p),
                                    ids.ctypes.data_as(C.POINTER(C.c_uint64)), len(ids),
                                    _ptr(out), _stream(stream)), self.handle)
        return out

    def callback_volume(self, vol_info, get_data):
        """get_data(node_id:int, dst:ctypes buffer address, nbytes:int) -> bool."""
        def _cb(user, node_id, dst, nbytes):
            try:
                return 0 if get_data(int(node_id), dst, int(nbytes)) else 1
            except Exception:
                return 1
        cfn = _abi.GET_DATA_FN(_cb)
        h = C.c_void_p()
        check(lib().lv_volume_create(self.handle, C.byref(vol_info.info), cfn, None,
                                     C.byref(h)), self.handle)
        return Volume(self, h, vol_info, keepalive=cfn)

    def open_volume(self, uri):
        """A volume from a data-source URI (mem://, raw://)."""
        h = C.c_void_p()
        check(lib().lv_volume_open(self.handle, uri.encode(), C.byref(h)), self.handle)
        info = _abi.VolumeInfo()
        check(lib().lv_volume_get_info(h, C.byref(info)))
        vi = VolumeInformation.__new__(VolumeInformation)
        vi.info = info
        return Volume(self, h, vi)

    def blob_bricks(self, vol_info, node_ids, n_blobs, seed, noise=0, stream=None):
        """Generated bricks of `node_ids` as a device tensor (n, brick_bytes) uint8."""
        import torch
        ids = np.ascontiguousarray(node_ids, np.uint64)
        out = torch.empty((len(ids), vol_info.brick_bytes), dtype=torch.uint8,
                          device=torch.device("cuda", self.device))
        d = _abi.BlobDesc(n_blobs, noise, seed)
        check(lib().lv_blob_generate(self.handle, C.byref(vol_info.info), C.byref(d),
                                     ids.ctypes.data_as(C.POINTER(C.c_uint64)), len(ids),
                                     _ptr(out), _stream(stream)), self.handle)
        return out

    def transfer_function(self, rgba):
        return TransferFunction(self, rgba)

    def purge(self):
        check(lib().lv_pool_purge(self.handle), self.handle)

    # -- rendering
    def render_desc(self, mv, proj, width, height, sse=1.0, min_lod=0, max_lod=100,
                    samples_per_ray=0, step_policy=STEP_HALF_VOXEL, early_exit=0.999,
                    filt=FILTER_TRILINEAR, data_range=(0.0, 0.0), synchronous=True,
                    max_uploads=1, time_step=0, clip_planes=None, rng=(0.0, 1.0), rect=None):
        """rect = (x, y, w, h): render only those pixels of the frame (a
        sort-first tile); None renders the whole frame."""
        d = _abi.RenderDesc()
        d.camera = make_camera(mv, proj)
        d.width, d.height = width, height
        d.lod = make_lod(height, sse, min_lod, max_lod, rng, time_step, clip_planes)
        d.samples_per_ray, d.step_policy, d.early_exit, d.filter = (
            samples_per_ray, step_policy, early_exit, filt)
        d.data_range[0], d.data_range[1] = data_range
        d.synchronous, d.max_uploads = int(bool(synchronous)), max_uploads
        if rect is not None:
            for i in range(4):
                d.rect[i] = int(rect[i])
        return d

    def render(self, volume, tf, desc, out=None, stream=None):
        """Renders one view into `out` (H, W, 4) float32 CUDA tensor."""
        import torch
        if out is None:
            out = torch.empty((desc.height, desc.width, 4), dtype=torch.float32,
                              device=torch.device("cuda", self.device))
        check(lib().lv_render(self.handle, volume.handle, tf.handle, C.byref(desc), _ptr(out),
                              _stream(stream)), self.handle)
        return out

    def write_png(self, frame, path):
        """Writes an (H, W, 4) float32 device frame as a PNG file."""
        H, W = frame.shape[:2]
        check(lib().lv_frame_write_png(self.handle, C.c_void_p(frame.data_ptr()), W, H,
                                       str(path).encode()), self.handle)

    def render_launch(self):
        """lv_render's ray-cast launch shape (lv_get_render_launch)."""
        c = _abi.RenderLaunch()
        check(lib().lv_get_render_launch(self.handle, C.byref(c)), self.handle)
        return {k: getattr(c, k) for k, _ in c._fields_}

    def set_render_launch(self, kind=_abi.LAUNCH_GRID, tile_w=8, tile_h=16,
                          samples_per_check=0, order=_abi.ORDER_RASTER, lookahead=0):
        """Ray-cast launch of lv_render: LAUNCH_GRID (tile = thread block),
        LAUNCH_TILE_QUEUE (resident CTAs over a tile queue) or
        LAUNCH_WARP_REFILL (warp tiles with lane refill); the queue kinds
        take tiles in ORDER_RASTER or ORDER_LONGEST_FIRST order; lookahead=1
        loads a ray's next sample before compositing the current one."""
        c = _abi.RenderLaunch(kind, tile_w, tile_h, samples_per_check, order, lookahead)
        check(lib().lv_set_render_launch(self.handle, C.byref(c)), self.handle)

    def frame_histogram(self, n_bins=256, data_range=(0.0, 255.0)):
        """Histogram of the last frame's bricks whose centre projects into the
        rendered rect (HistogramFilter's per-view histogram)."""
        acc = np.zeros(n_bins, np.uint64)
        check(lib().lv_frame_histogram(self.handle, n_bins, float(data_range[0]),
                                       float(data_range[1]),
                                       acc.ctypes.data_as(C.POINTER(C.c_uint64))), self.handle)
        return acc

    def totals(self):
        """Running totals of lv_render (frames, bricks and bytes streamed,
        launches) without waiting for the device."""
        t = _abi.CtxTotals()
        check(lib().lv_get_totals(self.handle, C.byref(t)), self.handle)
        return t.as_dict()

    def last_stats(self):
        s = _abi.FrameStats()
        check(lib().lv_last_stats(self.handle, C.byref(s)), self.handle)
        return s.as_dict()

    def to_rgba8(self, rgba, out=None, stream=None):
        import torch
        h, w = rgba.shape[:2]
        if out is None:
            out = torch.empty((h, w, 4), dtype=torch.uint8, device=rgba.device)
        check(lib().lv_frame_to_rgba8(self.handle, _ptr(rgba), w, h, _ptr(out),
                                      _stream(stream)), self.handle)
        return out


class Batch:
    """Batched renderer (lv_batch): many views per persistent launch, replayed
    as a CUDA graph."""

    def __init__(self, ctx):
        self.ctx = ctx
        h = C.c_void_p()
        check(lib().lv_batch_create(ctx.handle, C.byref(h)), ctx.handle)
        self.handle = h
        ctx._children.add(self)
        self._views = None

    def close(self):
        if self.handle:
            lib().lv_batch_destroy(self.handle)
            self.handle = None
            self.ctx._children.discard(self)

    def __del__(self):
        if sys.is_finalizing():
            return  # CUDA may already be torn down; the OS reclaims everything
        try:
            self.close()
        except Exception:
            pass

    def config(self):
        c = _abi.BatchConfig()
        check(lib().lv_batch_get_config(self.handle, C.byref(c)), self.ctx.handle)
        return c.as_dict()

    def set_config(self, tile_w=8, tile_h=16, ctas_per_sm=0, tf_shared=0, use_graph=1,
                   queue=_abi.QUEUE_CTA_TILES, samples_per_check=8, order=None,
                   lookahead=None):
        """order: ORDER_LONGEST_FIRST (default for CTA tiles) or ORDER_RASTER
        (the only order of warp refill); lookahead (view kernels only, 0 or
        1): default 0."""
        if order is None:
            order = (_abi.ORDER_RASTER if queue == _abi.QUEUE_WARP_REFILL
                     else _abi.ORDER_LONGEST_FIRST)
        if lookahead is None:
            lookahead = 0
        c = _abi.BatchConfig(tile_w, tile_h, ctas_per_sm, tf_shared, use_graph, queue,
                             samples_per_check, order, lookahead)
        check(lib().lv_batch_set_config(self.handle, C.byref(c)), self.ctx.handle)

    @staticmethod
    def _pack(items):
        """items: sequence of (Volume, TransferFunction, RenderDesc, out tensor)."""
        arr = (_abi.BatchView * len(items))()
        for i, (vol, tf, desc, out) in enumerate(items):
            arr[i].volume = vol.handle.value
            arr[i].tf = tf.handle.value
            arr[i].desc = desc
            arr[i].d_rgba = out.data_ptr()
        return arr

    def render(self, items, stream=None):
        arr = self._pack(items)
        self._views = (arr, items)  # keep tensors alive until the next call
        check(lib().lv_batch_render(self.handle, arr, len(items), _stream(stream)),
              self.ctx.handle)

    def graph_stats(self):
        """(captures, replays, cached graphs) of this batch's graph cache."""
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint32()
        check(lib().lv_batch_graph_stats(self.handle, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def stats(self, n):
        out = (_abi.FrameStats * max(n, 1))()
        sel, ray = C.c_float(), C.c_float()
        check(lib().lv_batch_stats(self.handle, out, n, C.byref(sel), C.byref(ray)),
              self.ctx.handle)
        return [out[i].as_dict() for i in range(n)], sel.value, ray.value

    def autotune(self, items, reps=3, stream=None):
        arr = self._pack(items)
        c = _abi.BatchConfig()
        check(lib().lv_batch_autotune(self.handle, arr, len(items), _stream(stream), reps,
                                      C.byref(c)), self.ctx.handle)
        return c.as_dict()

    def autotune_results(self):
        """[(config dict, mean ray-cast ms)] of every configuration the last
        autotune ran."""
        n = C.c_uint32()
        check(lib().lv_batch_autotune_results(self.handle, None, None, 0, C.byref(n)))
        cfgs = (_abi.BatchConfig * max(n.value, 1))()
        ms = (C.c_float * max(n.value, 1))()
        check(lib().lv_batch_autotune_results(self.handle, cfgs, ms, n.value, C.byref(n)))
        return [(cfgs[i].as_dict(), float(ms[i])) for i in range(n.value)]


class Server:
    """Render server (lv_server): continuous batching or plain per-request."""

    def __init__(self, ctx, mode=_abi.SERVE_BATCHED, max_batch=32, max_queue=0, use_graph=1,
                 tile=None, ctas_per_sm=0, max_pixels=0):
        self.ctx = ctx
        tw, th = tile if tile else (0, 0)
        cfg = _abi.ServerConfig(mode, max_batch, max_queue, use_graph, tw, th, ctas_per_sm,
                                max_pixels)
        h = C.c_void_p()
        check(lib().lv_server_create(ctx.handle, C.byref(cfg), C.byref(h)), ctx.handle)
        self.handle = h
        ctx._children.add(self)
        self._outs = {}

    def submit(self, volume, tf, desc, out):
        r = _abi.Request(volume.handle.value, tf.handle.value, desc, out.data_ptr())
        t = C.c_uint64()
        check(lib().lv_server_submit(self.handle, C.byref(r), C.byref(t)), self.ctx.handle)
        self._outs[t.value] = out
        return t.value

    def wait(self, ticket, timeout_ms=60000):
        res = _abi.RequestResult()
        st = lib().lv_server_wait(self.handle, ticket, timeout_ms, C.byref(res))
        check(st, self.ctx.handle)
        self._outs.pop(ticket, None)
        return {"status": res.status, "batch_size": res.batch_size,
                "latency_ms": res.latency_ms, "queue_ms": res.queue_ms,
                "stats": res.stats.as_dict()}

    def counters(self):
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        check(lib().lv_server_counters(self.handle, C.byref(a), C.byref(b), C.byref(c)))
        return {"completed": a.value, "batches": b.value, "queued": c.value}

    def profile(self):
        """Where the server thread's time went (lv_server_get_profile)."""
        p = _abi.ServerProfile()
        check(lib().lv_server_get_profile(self.handle, C.byref(p)))
        return {k: getattr(p, k) for k, _ in _abi.ServerProfile._fields_}

    def close(self):
        if self.handle:
            lib().lv_server_destroy(self.handle)
            self.handle = None
            self.ctx._children.discard(self)

    def __del__(self):
        if sys.is_finalizing():
            return  # CUDA may already be torn down; the OS reclaims everything
        try:
            self.close()
        except Exception:
            pass
