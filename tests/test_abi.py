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


def test_c_program_against_the_abi(tmp_path):
    """tests/cpp/abi_check.c: the header compiles as C11 (-pedantic -Werror),
    links against the library, and every entry point answers null or
    out-of-range arguments with its documented status without a device;
    tg_read_input reads a file and reports a short buffer and a missing file."""
    import shutil
    import subprocess

    import pytest
    if not shutil.which("gcc"):
        pytest.skip("gcc not found")
    lib = B.gpu_lib()
    exe = str(tmp_path / "abi_check")
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-pedantic", "-Werror",
                        "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "abi_check.c"),
                        "-o", exe, "-L", os.path.dirname(lib), "-ltuna_gpu", "-Wl,-rpath," + os.path.dirname(lib)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    inp = tmp_path / "in.fa"
    inp.write_bytes(b">a\nACGTA\n")
    r = subprocess.run([exe, str(inp)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr


def test_ctypes_structs_match_the_header(tmp_path):
    """The ctypes mirrors of tg_ctx_opts, tg_job_opts and tg_stats have the C
    header's size and field offsets (a C program prints them; a field name the
    header lacks does not compile)."""
    import json
    import shutil
    import subprocess

    import pytest
    import tuna_gb300 as T
    if not shutil.which("gcc"):
        pytest.skip("gcc not found")
    structs = {"tg_ctx_opts": T._CtxOpts, "tg_job_opts": T._JobOpts, "tg_stats": T._Stats}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "tuna_gpu.h"', "int main(void) {",
             '    printf("{");']
    for i, (name, cls) in enumerate(structs.items()):
        lines.append(f'    printf("{"," if i else ""}\\"{name}\\": [%zu", sizeof({name}));')
        for f, _ in cls._fields_:
            lines.append(f'    printf(", %zu", offsetof({name}, {f}));')
        lines.append('    printf("]");')
    lines += ['    printf("}\\n");', "    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = str(tmp_path / "layout")
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = json.loads(subprocess.run([exe], capture_output=True, text=True, check=True).stdout)
    for name, cls in structs.items():
        want = [ctypes.sizeof(cls)] + [getattr(cls, f).offset for f, _ in cls._fields_]
        assert got[name] == want, name
