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


def test_status_names_and_constants_match_the_header():
    """The binding's status names and constants are the header's."""
    text = open(os.path.join(ROOT, "include", "lantern_gpu.h")).read()
    enum = re.search(r"typedef enum lt_status \{(.*?)\} lt_status;", text, re.S).group(1)
    values = {int(v): n for n, v in re.findall(r"\b(LT_\w+)\s*=\s*(\d+)", enum)}
    assert values == native.STATUS
    consts = dict(re.findall(r"#define (LT_\w+) (\d+)u?\b", text))
    assert int(consts["LT_ABI_VERSION"]) == native.ABI_VERSION
    assert int(consts["LT_MAX_BATCH"]) == native.MAX_BATCH
    assert int(consts["LT_NOALLOC_MAX_PATHS"]) == native.NOALLOC_MAX_PATHS
    fields = re.search(r"typedef struct lt_queue_lengths \{(.*?)\} lt_queue_lengths;", text, re.S).group(1)
    assert re.findall(r"uint32_t (\w+);", fields) == [f for f, _ in native.QueueLengths._fields_]
