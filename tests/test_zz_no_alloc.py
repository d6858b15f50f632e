"""tvk_brick_lod0_noalloc: bricking for callers that cannot allocate device
memory at call time (a host with a fixed device-memory budget, work recorded
into a stream capture, a pre-sized pool).  The entry point keeps its
accumulators in a fixed array inside the library; this test gives it device
inputs and outputs that the test allocates itself, calls it twice in a row
with different bricks (the second call must not see the first call's
accumulators), and checks every output against the regular, allocating
path (tvk_volume_create + tvk_volume_get_brick / _get_minmax /
_get_brick_histograms): integer results, so bit for bit.

The file sorts last so a run that stops at the first failure has already run
every other test.
"""
import ctypes as C

import numpy as np
import pytest

from tuvok_gb300 import Volume
from tuvok_gb300 import _native as N
from tuvok_gb300.workloads import numpy_blob_volume

pytestmark = pytest.mark.gpu


class MinMax4(C.Structure):
    _fields_ = [("v", C.c_double * 4)]


def run_noalloc(torch, d_raw, dtype, dims, bs, ov, clamp, coords, shift, stream):
    lib = N.lib()
    sizes = []
    counts = [-(-dims[a] // (bs - 2 * ov)) for a in range(3)]
    for c in coords:
        s = []
        for a in range(3):
            core = bs - 2 * ov
            last = c[a] == counts[a] - 1
            s.append(2 * ov + dims[a] % core if (last and dims[a] % core) else bs)
        sizes.append(s)
    nvox = sum(s[0] * s[1] * s[2] for s in sizes)
    item = 1 if dtype == np.uint8 else 2
    out = torch.zeros(nvox * item, dtype=torch.uint8, device="cuda")
    mm = torch.zeros(len(coords) * 4, dtype=torch.float64, device="cuda")
    hist = torch.zeros(len(coords) * 256, dtype=torch.int32, device="cuda")
    flat = (C.c_uint64 * (3 * len(coords)))(*[int(v) for c in coords for v in c])
    st = lib.tvk_brick_lod0_noalloc(
        C.c_void_p(d_raw.data_ptr()), 0 if dtype == np.uint8 else 1,
        (C.c_uint64 * 3)(*dims), (C.c_uint32 * 3)(bs, bs, bs), ov, int(clamp), flat,
        len(coords), shift, C.c_void_p(out.data_ptr()), out.numel(),
        C.c_void_p(mm.data_ptr()), C.c_void_p(hist.data_ptr()), C.c_void_p(stream))
    N.check(st)
    torch.cuda.synchronize()
    host = out.cpu().numpy().view(dtype)
    bricks, o = [], 0
    for s in sizes:
        n = s[0] * s[1] * s[2]
        bricks.append(host[o:o + n].reshape(s[2], s[1], s[0]))
        o += n
    return bricks, mm.cpu().numpy().reshape(-1, 4), hist.cpu().numpy().reshape(-1, 256)


@pytest.mark.parametrize("dims,dtype,bs,ov,clamp", [
    ((61, 47, 39), np.uint16, 18, 1, False),
    ((40, 33, 20), np.uint8, 12, 2, True),
    # 10 x 10 x 10 bricks: both calls fill the array (exactly 64 bricks each)
    ((80, 80, 80), np.uint16, 12, 2, False),
])
def test_noalloc_matches_allocating_path_twice(cuda_ok, dims, dtype, bs, ov, clamp):
    import torch
    vmax = 255 if dtype == np.uint8 else 4095
    raw = numpy_blob_volume(dims, dtype, 7, (3, 9), (vmax * 0.3, vmax * 0.95), vmax, seed=31,
                            noise=3)
    ref = Volume(raw, brick_size=(bs, bs, bs), overlap=ov, clamp_to_edge=clamp)
    ref_hist, shift = ref.GetBrickHistograms()
    layout = ref.GetBrickLayout(0)
    all_coords = [(x, y, z) for z in range(layout[2]) for y in range(layout[1])
                  for x in range(layout[0])]
    d_raw = torch.from_numpy(raw.reshape(-1).view(np.uint8).copy()).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row over different (and differently sized) brick sets
    first = all_coords[::2][:N_MAX]
    second = all_coords[1::2][:N_MAX][::-1]
    if len(all_coords) >= 2 * N_MAX:
        assert len(first) == len(second) == N_MAX
    for coords in (first, second):
        bricks, mm, hist = run_noalloc(torch, d_raw, dtype, dims, bs, ov, clamp, coords, shift,
                                       stream)
        for b, c in enumerate(coords):
            k = ref.IndexFrom4D(c[0], c[1], c[2], 0)
            np.testing.assert_array_equal(bricks[b], ref.GetBrick((0, 0, k)), err_msg=str(c))
            m = ref.MaxMinForKey((0, 0, k))
            assert tuple(mm[b]) == (m.min_scalar, m.max_scalar, m.min_gradient, m.max_gradient)
            np.testing.assert_array_equal(hist[b].astype(np.uint32), ref_hist[k])


N_MAX = 64


def test_noalloc_rejects_too_many_bricks(cuda_ok):
    import torch
    lib = N.lib()
    d = torch.zeros(16, dtype=torch.uint8, device="cuda")
    coords = (C.c_uint64 * (3 * 65))()
    st = lib.tvk_brick_lod0_noalloc(C.c_void_p(d.data_ptr()), 0, (C.c_uint64 * 3)(2, 2, 2),
                                    (C.c_uint32 * 3)(4, 4, 4), 1, 0, coords, 65, 0,
                                    C.c_void_p(d.data_ptr()), 16, C.c_void_p(d.data_ptr()),
                                    C.c_void_p(d.data_ptr()), None)
    assert st == 1 and b"1..64" in lib.tvk_last_error()
    st = lib.tvk_brick_lod0_noalloc(C.c_void_p(d.data_ptr()), 0, (C.c_uint64 * 3)(8, 8, 8),
                                    (C.c_uint32 * 3)(6, 6, 6), 1, 0, (C.c_uint64 * 3)(0, 0, 0),
                                    1, 0, C.c_void_p(d.data_ptr()), 16,
                                    C.c_void_p(d.data_ptr()), C.c_void_p(d.data_ptr()), None)
    assert st == 1 and b"output buffer" in lib.tvk_last_error()
    # misaligned outputs are refused before any GPU work
    base = d.data_ptr()
    for args, what in (((base + 1, base, base), b"voxel pointers"),
                       ((base, base + 4, base), b"8-byte"),
                       ((base, base, base + 2), b"4-byte")):
        out, mm, hist = args
        st = lib.tvk_brick_lod0_noalloc(C.c_void_p(base), 1, (C.c_uint64 * 3)(4, 4, 4),
                                        (C.c_uint32 * 3)(6, 6, 6), 1, 0, (C.c_uint64 * 3)(0, 0, 0),
                                        1, 0, C.c_void_p(out), 1 << 20, C.c_void_p(mm),
                                        C.c_void_p(hist), None)
        assert st == 1 and what in lib.tvk_last_error(), what
