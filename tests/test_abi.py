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
