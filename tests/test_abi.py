"""The C-ABI library loads and exports every function include/lantern_gpu.h
declares (no GPU needed; nothing is called that touches a device)."""
import ctypes
import os
import re

from lantern_gb300 import build, native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            text = open(os.path.join(ROOT, "include", f)).read()
            names |= set(re.findall(r"^\w[\w\s\*]*?\b(lt_\w+)\s*\(", text, re.M))
    return names


def test_library_exports_every_declared_symbol():
    """Both builds: the library and its bound-checked twin."""
    build.build()
    declared = _declared()
    assert declared, "no declarations found"
    for path in (build.LIB, build.CHECKED_LIB):
        lib = ctypes.CDLL(path)
        missing = [n for n in sorted(declared) if not hasattr(lib, n)]
        assert not missing, (path, missing)
    assert set(native.SYMBOLS) <= declared


def test_abi_version_and_no_device_error():
    lib = native.load()
    assert lib.lt_abi_version() == native.ABI_VERSION
    import torch
    if not torch.cuda.is_available():
        h = ctypes.c_void_p()
        st = lib.lt_ctx_create(0, ctypes.byref(h))
        assert st != 0 and lib.lt_last_error(None)
