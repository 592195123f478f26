"""The C-ABI library loads and exports every entry point include/*.h declares
(no GPU needed; no compute calls are made)."""
import ctypes
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(lv_[a-z0-9_]+)\s*\((?!\*)", text):  # not "T (*fn)("
            names.add(m.group(1))
    return names


def test_all_declared_symbols_exported(native):
    syms = declared_symbols()
    assert "lv_render" in syms and "lv_select_visible" in syms
    missing = [s for s in sorted(syms) if not hasattr(native, s)]
    assert not missing, missing


def test_abi_version(native):
    assert native.lv_abi_version() == 1


def test_ctx_create_rejects_bad_device(native):
    import livre_gb300._abi as abi
    h = ctypes.c_void_p()
    assert native.lv_ctx_create(-1, ctypes.byref(h)) == abi.LV_EDEVICE
    assert not h.value


def test_null_arguments_rejected(native):
    import livre_gb300._abi as abi
    assert native.lv_fill_regular_volume_info(None) == abi.LV_EINVAL
    info = abi.VolumeInfo()
    assert native.lv_fill_regular_volume_info(ctypes.byref(info)) == abi.LV_EINVAL  # 0 voxels


def test_product_never_imports_oracle():
    """The product package and the C sources do not reference the oracle."""
    for path in glob.glob(os.path.join(ROOT, "livre_gb300", "**", "*"), recursive=True):
        if os.path.isfile(path) and path.endswith((".py", ".cu", ".h", ".cpp")):
            text = open(path).read()
            assert "pyoracle" not in text and "oracle/" not in text and "or_" + "raycast" not in text, path


def test_brick_slot_bytes_by_layout(native):
    """Pool bytes per brick (lv_brick_slot_bytes with no context: the default
    layout). uint8 bricks of 64 to 1024 voxels per row are voxel quads: the
    canonical bytes staged at three times the voxel count (256-byte
    aligned), the slot rounded to whole 1 KiB units; every other brick keeps
    one element per voxel. Host arithmetic only, no device call."""
    import livre_gb300 as lv

    def kib(b):
        return (b + 1023) // 1024 * 1024

    for voxels, block, overlap, dtype, quads in [
            (2048, 64, 1, lv.DT_UINT8, True),     # 66^3: the 2048^3 headline bricks
            (256, 128, 1, lv.DT_UINT8, True),     # 130^3
            (256, 62, 1, lv.DT_UINT8, True),      # 64^3: the smallest quad row
            (256, 32, 1, lv.DT_UINT8, False),     # 34^3: compact (rows under 64)
            (1024, 128, 1, lv.DT_UINT16, False),  # uint16 stays compact
    ]:
        vi = lv.VolumeInformation(voxels, block, overlap, dtype=dtype)
        n = (block + 2 * overlap) ** 3 * (2 if dtype == lv.DT_UINT16 else 1)
        want = kib((3 * n + 255) // 256 * 256 + n) if quads else kib(n)
        assert vi.slot_bytes == want, (voxels, block, dtype, vi.slot_bytes, want)
