"""A C++ host (tests/cpp/shim_demo.cpp over include/tvk_renderer.hpp) links
the library, paints a frame with the ray caster and a converged GridLeaper
frame, and gets images bit-identical to the same calls through the Python
binding."""
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from tuvok_gb300 import Pool, Renderer, Volume
from tuvok_gb300 import _native as N

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def fnv1a(a):
    h = 1469598103934665603
    for b in np.ascontiguousarray(a).tobytes():
        h ^= b
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def demo_volume():
    z, y, x = np.meshgrid(np.arange(40), np.arange(48), np.arange(64), indexing="ij")
    v = 255 - ((x - 30) ** 2 + (y - 22) ** 2 + (z - 19) ** 2) // 3
    return np.clip(v, 0, 255).astype(np.uint8)


def demo_tf():
    i = np.arange(256)
    f = np.float32
    t = np.zeros((256, 4), dtype=np.float32)
    t[:, 0] = i.astype(f) / f(255.0)
    t[:, 1] = f(0.8) * t[:, 0]
    t[:, 2] = f(1.0) - t[:, 0]
    t[:, 3] = np.where(i < 40, f(0.0), (f(0.6) * (i - 40).astype(f)) / f(215.0))
    return t


def test_gpu_cpp_host_matches_python_binding(cuda_ok, tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    lib_dir = Path(N.LIB_PATH).resolve().parent
    exe = tmp_path / "shim_demo"
    subprocess.run([gxx, "-std=c++17", "-O2", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "cpp" / "shim_demo.cpp"), "-o", str(exe),
                    f"-L{lib_dir}", "-ltvk", f"-Wl,-rpath,{lib_dir}",
                    "-L/usr/local/cuda/lib64", "-Wl,-rpath,/usr/local/cuda/lib64"],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = dict(re.findall(r"(\w+)=(\S+)", out))

    vol = Volume(demo_volume(), brick_size=(18, 18, 18), overlap=1)
    r = Renderer()
    r.RegisterDataset(vol)
    r.Set1DTransFloat(demo_tf())
    r.SetUseLighting(True)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=(0.4, 0.5, 1.4))
    r.Resize(96, 64)
    r.Paint()
    assert int(got["plain_fnv"], 16) == fnv1a(r.ReadBackPixels())
    assert int(got["samples"]) == r.GetStats().samples
    pool = Pool(vol, 1 << 30)
    info = pool.Paint(r, max_passes=64)
    assert int(got["leaper_fnv"], 16) == fnv1a(r.ReadBackPixels())
    assert int(got["passes"]) == info.passes and int(got["converged"]) == info.converged == 1
    assert int(got["lods"]) == vol.GetLODLevelCount()
