"""The C ABI library loads and exports every entry point of include/tuna_gpu.h
(no GPU needed: nothing is called that touches a device)."""
import ctypes
import os
import re

from tuna_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    with open(os.path.join(ROOT, "include", "tuna_gpu.h")) as f:
        src = f.read()
    return sorted(set(re.findall(r"\b(tg_[a-z_]+)\s*\(", src)) - {"tg_sink_fn", "tg_part_sink_fn", "tg_status"})


def test_library_exports_every_declared_symbol():
    path = B.gpu_lib()
    lib = ctypes.CDLL(path)
    missing = [s for s in _declared() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_front_end_lists_the_abi():
    import tuna_gb300 as T
    assert set(T.ABI_SYMBOLS) == set(_declared())


def test_version_and_device_count_without_gpu():
    lib = ctypes.CDLL(B.gpu_lib())
    lib.tg_version.restype = ctypes.c_char_p
    assert b"tuna-gb300" in lib.tg_version()
    lib.tg_device_count.restype = ctypes.c_int
    assert lib.tg_device_count() >= 0
