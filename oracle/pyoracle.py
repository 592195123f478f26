"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, as the checker. The product package livre_gb300 never does.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build


class Volume(C.Structure):
    _fields_ = [("voxels", C.c_uint32 * 3), ("max_block", C.c_uint32 * 3),
                ("overlap", C.c_uint32 * 3), ("wspv", C.c_float),
                ("world_size", C.c_float * 3), ("depth", C.c_uint32),
                ("root_blocks", C.c_uint32 * 3)]


class Frustum(C.Structure):
    _fields_ = [("inv_mv", C.c_float * 16), ("inv_p", C.c_float * 16),
                ("left", C.c_float), ("right", C.c_float), ("bottom", C.c_float),
                ("top", C.c_float), ("nearp", C.c_float), ("farp", C.c_float),
                ("planes", (C.c_float * 4) * 6), ("eye", C.c_float * 3),
                ("dir", C.c_float * 3)]


class BlobParams(C.Structure):
    _fields_ = [("n_blobs", C.c_uint32), ("noise", C.c_uint32),
                ("dtype", C.c_uint32), ("seed", C.c_uint64)]


class FbmParams(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("octaves", C.c_uint32), ("lacunarity", C.c_float),
                ("gain", C.c_float), ("frequency", C.c_float), ("dtype", C.c_uint32)]


class View(C.Structure):
    _fields_ = [("mv", C.c_float * 16), ("proj", C.c_float * 16),
                ("width", C.c_uint32), ("height", C.c_uint32),
                ("n_samples", C.c_uint32), ("alpha_correction", C.c_float),
                ("early_exit", C.c_float), ("range_lo", C.c_float),
                ("range_hi", C.c_float), ("filter", C.c_uint32),
                ("n_clip", C.c_uint32), ("clip", (C.c_float * 4) * 6)]


MODE_PER_RAY = 0
MODE_SHADER = 1
ACCUMULATE = 0x100  # flag: rays start from the colour already in `out`
QUANT_WEIGHTS = 0x200  # flag: trilinear weights rounded to 1/256 (texture-unit filter)

# per-pixel flags of raycast(..., diagnostics=True) in shader mode
PX_DUPLICATE = 1  # a face grid point sampled by the bricks on both sides
PX_INVERTED = 2   # a nearer brick composited after a farther one
PX_GAP = 4        # a face grid point sampled by neither brick

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.or_fill_regular_volume_info.argtypes = [C.POINTER(Volume)]
        L.or_node_world_box.argtypes = [C.POINTER(Volume), C.c_uint64, C.POINTER(C.c_float)]
        L.or_node_children.argtypes = [C.c_uint64, C.POINTER(C.c_uint64)]
        L.or_frustum_setup.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(Frustum)]
        L.or_select_visible.argtypes = [
            C.POINTER(Volume), C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_uint32,
            C.c_float, C.c_uint32, C.c_uint32, C.POINTER(C.c_float), C.POINTER(C.c_float),
            C.c_uint32, C.c_uint32, C.POINTER(C.c_uint64), C.c_uint32,
            C.POINTER(C.c_uint32), C.POINTER(C.c_uint64)]
        L.or_default_tf.argtypes = [C.POINTER(C.c_float)]
        L.or_tf_lut.argtypes = [C.POINTER(C.c_float), C.c_uint32, C.POINTER(C.c_uint8)]
        L.or_blob_brick.argtypes = [C.POINTER(Volume), C.POINTER(BlobParams), C.c_uint64, C.c_void_p]
        L.or_blob_value.argtypes = [C.POINTER(Volume), C.POINTER(BlobParams), C.c_float, C.c_float, C.c_float]
        L.or_blob_value.restype = C.c_float
        L.or_fbm_brick.argtypes = [C.POINTER(Volume), C.POINTER(FbmParams), C.c_uint64,
                                   C.c_void_p]
        L.or_perlin.argtypes = [C.c_uint64, C.c_float, C.c_float, C.c_float]
        L.or_perlin.restype = C.c_float
        L.or_exp_neg.argtypes = [C.c_float]
        L.or_exp_neg.restype = C.c_float
        L.or_raycast.argtypes = [
            C.POINTER(Volume), C.c_uint32, C.POINTER(C.c_uint64), C.c_uint32, C.c_void_p,
            C.POINTER(C.c_float), C.c_uint32, C.POINTER(View), C.c_int, C.c_int,
            C.c_uint32, C.c_uint32, C.POINTER(C.c_double), C.POINTER(C.c_uint64)]
        L.or_raycast_px.argtypes = L.or_raycast.argtypes + [C.c_void_p, C.c_void_p]
        _lib = L
    return _lib


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def volume(voxels, block, overlap=0):
    """VolumeInformation for a regular volume (maximumBlockSize = block + 2*overlap)."""
    v = Volume()
    for i in range(3):
        v.voxels[i] = int(voxels[i] if hasattr(voxels, "__len__") else voxels)
        b = block[i] if hasattr(block, "__len__") else block
        o = overlap[i] if hasattr(overlap, "__len__") else overlap
        v.overlap[i] = int(o)
        v.max_block[i] = int(b) + 2 * int(o)
    if lib().or_fill_regular_volume_info(C.byref(v)) != 0:
        raise ValueError("invalid volume")
    return v


def world_box(vol, node_id):
    out = (C.c_float * 6)()
    lib().or_node_world_box(C.byref(vol), C.c_uint64(node_id), out)
    return np.array(out, dtype=np.float32)


def children(node_id):
    out = (C.c_uint64 * 8)()
    lib().or_node_children(C.c_uint64(node_id), out)
    return list(out)


def frustum(mv, proj):
    mv = np.ascontiguousarray(mv, dtype=np.float32).reshape(16)
    proj = np.ascontiguousarray(proj, dtype=np.float32).reshape(16)
    f = Frustum()
    if lib().or_frustum_setup(_fptr(mv), _fptr(proj), C.byref(f)) != 0:
        raise ValueError("singular matrix")
    return f


def select_visible(vol, mv, proj, window_height, sse, min_lod=0, max_lod=100,
                   rng=(0.0, 1.0), clip_planes=None, time_step=0, capacity=1 << 22):
    mv = np.ascontiguousarray(mv, dtype=np.float32).reshape(16)
    proj = np.ascontiguousarray(proj, dtype=np.float32).reshape(16)
    r = np.array(rng, dtype=np.float32)
    cp = np.zeros((6, 4), np.float32) if clip_planes is None else np.ascontiguousarray(clip_planes, np.float32)
    ncp = 0 if clip_planes is None else len(clip_planes)
    out = np.zeros(capacity, dtype=np.uint64)
    n = C.c_uint32()
    visited = C.c_uint64()
    rc = lib().or_select_visible(C.byref(vol), _fptr(mv), _fptr(proj), window_height, sse,
                                 min_lod, max_lod, _fptr(r), _fptr(cp), ncp, time_step,
                                 out.ctypes.data_as(C.POINTER(C.c_uint64)), capacity,
                                 C.byref(n), C.byref(visited))
    if rc != 0:
        raise RuntimeError("or_select_visible failed: %d" % rc)
    return out[: n.value].copy(), visited.value


def default_tf():
    out = np.zeros(256 * 4, np.float32)
    lib().or_default_tf(_fptr(out))
    return out.reshape(256, 4)


def tf_lut(rgba):
    rgba = np.ascontiguousarray(rgba, np.float32)
    n = rgba.shape[0]
    out = np.zeros(n * 4, np.uint8)
    lib().or_tf_lut(_fptr(rgba), n, out.ctypes.data_as(C.POINTER(C.c_uint8)))
    return out.reshape(n, 4)


def blob_params(n_blobs, seed, noise=0, dtype=1):
    p = BlobParams()
    p.n_blobs, p.noise, p.dtype, p.seed = n_blobs, noise, dtype, seed
    return p


def blob_brick(vol, bp, node_id):
    n = vol.max_block[0] * vol.max_block[1] * vol.max_block[2]
    out = np.zeros(n, np.uint16 if bp.dtype == 2 else np.uint8)
    if lib().or_blob_brick(C.byref(vol), C.byref(bp), C.c_uint64(node_id), out.ctypes.data) != 0:
        raise ValueError("bad node")
    return out


def fbm_params(seed, octaves=6, lacunarity=2.0, gain=0.5, frequency=8.0, dtype=2):
    p = FbmParams()
    p.seed, p.octaves, p.lacunarity, p.gain, p.frequency, p.dtype = (
        seed, octaves, lacunarity, gain, frequency, dtype)
    return p


def fbm_brick(vol, fp, node_id):
    n = vol.max_block[0] * vol.max_block[1] * vol.max_block[2]
    out = np.zeros(n, np.uint16 if fp.dtype == 2 else np.uint8)
    if lib().or_fbm_brick(C.byref(vol), C.byref(fp), C.c_uint64(node_id), out.ctypes.data) != 0:
        raise ValueError("bad node")
    return out


def perlin(seed, x, y, z):
    return lib().or_perlin(seed, float(x), float(y), float(z))


def exp_neg(x):
    return lib().or_exp_neg(float(x))


def make_view(mv, proj, width, height, n_samples, alpha_correction=None,
              early_exit=0.999, range_lo=0.0, range_hi=255.0, filt=1, clip_planes=None):
    v = View()
    for i, x in enumerate(np.asarray(mv, np.float32).reshape(16)):
        v.mv[i] = float(x)
    for i, x in enumerate(np.asarray(proj, np.float32).reshape(16)):
        v.proj[i] = float(x)
    v.width, v.height, v.n_samples = width, height, n_samples
    v.alpha_correction = (32.0 / n_samples) if alpha_correction is None else alpha_correction
    v.early_exit, v.range_lo, v.range_hi, v.filter = early_exit, range_lo, range_hi, filt
    if clip_planes is not None:
        v.n_clip = len(clip_planes)
        for i, pl in enumerate(clip_planes):
            for j in range(4):
                v.clip[i][j] = float(pl[j])
    return v


def raycast(vol, dtype, node_ids, bricks, tf, view, mode=MODE_PER_RAY, n_threads=0,
            rows=None, init=None, diagnostics=False):
    """init: an image to composite behind (mode | ACCUMULATE is implied).
    diagnostics: also return per-pixel sample counts (uint32) and flags
    (uint8, PX_* bits, shader mode only) as (image, n_samples, counts, flags)."""
    ids = np.ascontiguousarray(node_ids, np.uint64)
    bricks = np.ascontiguousarray(bricks)
    tf = np.ascontiguousarray(tf, np.float32).reshape(-1, 4)
    if init is None:
        out = np.zeros((view.height, view.width, 4), np.float64)
    else:
        out = np.array(init, np.float64, copy=True, order="C")
        mode |= ACCUMULATE
    r0, r1 = (0, view.height) if rows is None else rows
    ns = C.c_uint64()
    counts = np.zeros((view.height, view.width), np.uint32)
    flags = np.zeros((view.height, view.width), np.uint8)
    rc = lib().or_raycast_px(C.byref(vol), dtype, ids.ctypes.data_as(C.POINTER(C.c_uint64)),
                             len(ids), bricks.ctypes.data, _fptr(tf), tf.shape[0],
                             C.byref(view), mode, n_threads, r0, r1,
                             out.ctypes.data_as(C.POINTER(C.c_double)), C.byref(ns),
                             counts.ctypes.data if diagnostics else None,
                             flags.ctypes.data if diagnostics else None)
    if rc != 0:
        raise RuntimeError("or_raycast failed: %d" % rc)
    if diagnostics:
        return out, ns.value, counts, flags
    return out, ns.value
