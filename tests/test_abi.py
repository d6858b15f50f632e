"""The C-ABI library loads and exports every entry point include/tvk.h declares,
and its argument checks answer before any GPU work (no GPU needed)."""
import ctypes as C
import re
from pathlib import Path

import pytest

from tuvok_gb300 import _native as N

HEADER = Path(__file__).resolve().parent.parent / "include" / "tvk.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(tvk_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_api():
    names = declared_functions()
    assert "tvk_paint" in names and "tvk_volume_create" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(N.LIB_PATH))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_binding_covers_the_header():
    assert set(declared_functions()) == set(N.PROTOTYPES)


def test_status_strings_and_version():
    lib = N.lib()
    assert lib.tvk_abi_version() == 1
    assert lib.tvk_status_string(0) == b"ok"
    assert lib.tvk_status_string(4) == b"unsupported"


def test_invalid_arguments_rejected_before_gpu_work():
    lib = N.lib()
    h = C.c_void_p()
    dims = (C.c_uint64 * 3)(8, 8, 8)
    bs = (C.c_uint32 * 3)(4, 4, 4)
    # null voxels
    assert lib.tvk_volume_create(None, 0, dims, bs, 1, 0, C.byref(h)) == 1
    assert b"null" in lib.tvk_last_error()
    buf = (C.c_uint8 * 512)()
    # brick not larger than twice the overlap (ExtendedOctree.cpp:196-198)
    assert lib.tvk_volume_create(buf, 0, dims, (C.c_uint32 * 3)(2, 2, 2), 1, 0, C.byref(h)) == 1
    # bad dtype
    assert lib.tvk_volume_create(buf, 7, dims, bs, 1, 0, C.byref(h)) == 1
    # null renderer handles
    assert lib.tvk_paint(None) == 1
    assert lib.tvk_set_sample_rate_modifier(None, 1.0) == 1
    assert lib.tvk_volume_destroy(None) == 0  # destroying nothing is fine


def test_check_raises_with_message():
    with pytest.raises(N.TvkError) as e:
        N.check(N.lib().tvk_paint(None))
    assert "TVK_ERR_INVALID_ARG" in str(e.value)


def test_cpp_shim_compiles():
    """include/tvk_renderer.hpp (the C++ mirror of AbstrRenderer, BrickedDataset,
    GLVolumePool) and the C++ host example compile against include/tvk.h."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    root = HEADER.parent.parent
    subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-Werror",
                    f"-I{root / 'include'}", str(root / "tests" / "cpp" / "shim_demo.cpp")],
                   check=True)

