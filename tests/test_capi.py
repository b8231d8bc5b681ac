"""The C ABI: the library builds, loads without a GPU, exports every symbol
include/enkfg.h declares, and reports errors by status code (no abort)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "enkfg.h")).read()
    return sorted(set(re.findall(r"ENKFG_API\s+[\w\s\*]+?\b(enkfg_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    import build
    path = build.build()
    return C.CDLL(path)


def test_header_lists_entry_points():
    syms = header_symbols()
    assert "enkfg_calc_transforms" in syms and "enkfg_update_fields" in syms and len(syms) >= 20


def test_exports_every_declared_symbol(lib):
    for s in header_symbols():
        assert hasattr(lib, s), s


def test_binding_covers_header():
    import enkfg
    assert sorted(enkfg.EXPORTS) == header_symbols()


def test_status_strings_and_errors_without_device(lib):
    lib.enkfg_status_string.restype = C.c_char_p
    assert lib.enkfg_status_string(0) == b"ok"
    assert lib.enkfg_status_string(8) == b"unsupported option"
    assert lib.enkfg_version() >= 1
    h = C.c_void_p()
    st = lib.enkfg_create(0, C.byref(h))
    if st != 0:                         # no GPU here: a status, not a crash
        assert h.value is None
    else:
        lib.enkfg_destroy(h)
    # calls on a NULL context fail cleanly
    assert lib.enkfg_standardise(None) == 1
    assert lib.enkfg_set_grid(None, None) == 1
    assert lib.enkfg_set_obstype_nlobsmax(None, 1, None) == 1
    assert lib.enkfg_set_obstype_visible(None, 1, None) == 1
    assert lib.enkfg_set_field_noise(None, 0, 0, None, None, None) == 1


def test_plain_c_client(tmp_path):
    """A C99 program that includes only enkfg.h and links libenkfg.so, as
    EnKF-C's host code would (tests/c_client.c)."""
    import shutil
    import subprocess
    import build
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = build.build()
    exe = tmp_path / "c_client"
    src = os.path.join(ROOT, "tests", "c_client.c")
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), src,
                        "-o", str(exe), "-L", os.path.dirname(lib), "-lenkfg", "-Wl,-rpath," + os.path.dirname(lib),
                        "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), str(tmp_path / "t.nc")], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
