"""Render parity on the benchmark's own configurations, at full size.

Each volume is generated on the GPU by tvk_generate_volume (the bytes checked
against the oracle's host restatement of the generator where that is cheap)
and rendered through the C ABI; the same bytes go to the oracle.  Every frame
(or every sampled row of a 1080p frame) is held to the FP32 oracle with the
usual bar -- per-pixel RGBA within 2/255, mean within 0.25/255, sample counts
equal pixel for pixel -- and the FP64 oracle's distance is printed per
configuration and held to the mean bar.

* plain, small: 256^3 uint8 (32 blobs + integer noise), 64^3 + 1 ghost voxel
  bricks, 512x512, sample-rate modifier 1.0, unlit, 3 orbit poses;
* plain, large, lit: 1024^3 uint16 12-bit (256 blobs + 3-octave value noise),
  128^3 + 1 bricks, 1920x1080, sample-rate modifier 1.5, Blinn-Phong and the
  reference lighting model, 2 poses, every 8th row;
* batching: views of the 2D TF of three Gaussian lobes in one batched paint
  over the 512^3 uint16 and 384x384x256 uint8 volumes, lit and unlit, sample
  rates 0.5 / 1 / 2;
* out-of-core LOD: the GridLeaper's isosurface (128, lit) over a 1024^3 uint8
  volume of 1024 blobs + 4-octave noise at 1920x1080, one pass over the
  converged brick cache, every 8th row.
"""
import numpy as np
import pytest

import oracle as O
from tuvok_gb300 import Batch, Pool, Renderer, Volume, generate_volume_device
from tuvok_gb300.workloads import (BATCH_VOLUMES, WORKLOADS, flythrough_poses, ooc_lod,
                                   tf2d_lobes)
from test_gpu_render import MAX_TOL, MEAN_TOL

pytestmark = pytest.mark.gpu


def device_volume(torch, w):
    """(device byte tensor, host [z, y, x] array) of workload w's volume."""
    n = w.dims[0] * w.dims[1] * w.dims[2] * np.dtype(w.dtype).itemsize
    d = torch.empty(n, dtype=torch.uint8, device="cuda")
    generate_volume_device(d.data_ptr(), w.dims, w.dtype, w.blobs(), w.noise_amp,
                           w.noise_octaves, w.noise_cell, w.seed, int(w.int_noise), w.vmax)
    torch.cuda.synchronize()
    host = d.cpu().numpy().view(w.dtype).reshape(w.dims[2], w.dims[1], w.dims[0])
    return d, host


def gpu_volume(d, w):
    return Volume(d.data_ptr(), brick_size=w.brick_size, overlap=w.overlap, dims=w.dims,
                  dtype=w.dtype)


def check_rows(img, cnt, ref, rc, rows, what):
    g, r = img[rows].astype(np.float64), ref[rows].astype(np.float64)
    d = np.abs(g - r)
    assert np.isfinite(g).all(), what
    assert d.max() <= MAX_TOL, f"{what}: max |diff| {d.max() * 255:.3f}/255"
    assert d.mean() <= MEAN_TOL, f"{what}: mean |diff| {d.mean() * 255:.4f}/255"
    if cnt is not None:
        off = int((cnt[rows] != rc[rows]).sum())
        assert off == 0, f"{what}: {off} pixels with other sample counts"
    return d


def fp64_report(img, ref64, rows, what):
    d = np.abs(img[rows].astype(np.float64) - ref64[rows].astype(np.float64))
    print(f"\n{what}: FP64 oracle distance max {d.max() * 255:.4f}/255, "
          f"mean {d.mean() * 255:.5f}/255 over {len(rows)} rows")
    assert d.mean() <= MEAN_TOL, what
    return d


def test_gpu_generator_equals_host_restatement(cuda_ok):
    """tvk_generate_volume and the oracle's restatement give the same bytes
    (integer noise, value noise of 3 and 4 octaves, uint8 and uint16)."""
    import torch
    cases = [WORKLOADS["plain_small"], BATCH_VOLUMES[1],
             ooc_lod(256), WORKLOADS["plain_medium_lit"]]
    for w in cases:
        d, host = device_volume(torch, w)
        ref = O.generate_volume(w.dims, w.dtype, w.blobs(), w.noise_amp, w.noise_octaves,
                                w.noise_cell, w.seed, int(w.int_noise), w.vmax)
        diff = int((host != ref).sum())
        assert diff == 0, f"{w.name}: {diff} voxels differ"
        assert O.volume_hash(host) == O.volume_hash(ref)
        assert host.max() > host.min()  # not an empty volume


def test_gpu_plain_small_full_size_matches_oracle(cuda_ok):
    import torch
    w = WORKLOADS["plain_small"]
    d, raw = device_volume(torch, w)
    vol = gpu_volume(d, w)
    r = Renderer()
    r.RegisterDataset(vol)
    r.Set1DTransFloat(w.tf())
    r.SetUseLighting(False)
    r.SetSampleRateModifier(w.srm)
    r.Resize(w.width, w.height)
    prep = O.Prepared(raw, w.brick_size, w.overlap, w.tf(), srm=w.srm, lighting=False)
    rows = np.arange(w.height)
    for k, (eye, at, up) in enumerate(w.poses(3)):
        r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye, at=at, up=up)
        r.Paint()
        img, cnt = r.ReadBackPixels(), r.ReadSampleCounts()
        ref, n, _, rc = prep.render(eye=eye, at=at, up=up, width=w.width, height=w.height,
                                    want_counts=True)
        check_rows(img, cnt, ref, rc, rows, f"plain_small pose {k}")
        assert r.GetStats().samples == n
        assert (img[..., 3] > 0).mean() > 0.2
        ref64, _, _ = prep.render(eye=eye, at=at, up=up, width=w.width, height=w.height,
                                  use_double=True)
        fp64_report(img, ref64, rows, f"plain_small pose {k}")
    prep.close()


@pytest.mark.parametrize("light_model", [1, 0], ids=["blinn_phong", "reference_light"])
def test_gpu_plain_large_lit_rows_match_oracle(cuda_ok, light_model):
    import torch
    w = WORKLOADS["plain_large_lit"]
    d, raw = device_volume(torch, w)
    vol = gpu_volume(d, w)
    r = Renderer()
    r.RegisterDataset(vol)
    r.Set1DTransFloat(w.tf())
    r.SetUseLighting(True)
    r.SetLightModel(light_model, 0.2, 0.6, 0.2, 32.0)
    r.SetSampleRateModifier(w.srm)
    r.Resize(w.width, w.height)
    prep = O.Prepared(raw, w.brick_size, w.overlap, w.tf(), srm=w.srm, lighting=True,
                      light_model=light_model)
    for k, (eye, at, up) in enumerate(w.poses(2)):
        r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye, at=at, up=up)
        r.Paint()
        img, cnt = r.ReadBackPixels(), r.ReadSampleCounts()
        ref, _, _, rc = prep.render(eye=eye, at=at, up=up, width=w.width, height=w.height,
                                    row_stride=8, want_counts=True)
        rows = np.arange(0, w.height, 8)
        check_rows(img, cnt, ref, rc, rows, f"plain_large_lit pose {k} model {light_model}")
        assert (img[rows, :, 3] > 0).mean() > 0.05
        ref64, _, _ = prep.render(eye=eye, at=at, up=up, width=w.width, height=w.height,
                                  row_stride=32, use_double=True)
        fp64_report(img, ref64, np.arange(0, w.height, 32),
                    f"plain_large_lit pose {k} model {light_model}")
    prep.close()


def test_gpu_batch_2d_lobes_views_match_oracle(cuda_ok):
    import torch
    tf = tf2d_lobes()
    vols = {}
    for idx in (2, 3):
        w = BATCH_VOLUMES[idx]
        d, raw = device_volume(torch, w)
        vols[idx] = (w, d, raw, gpu_volume(d, w))
    # volume, (w, h), srm, lit
    views = [(3, (1024, 1024), 2.0, True), (2, (1280, 720), 0.5, False),
             (3, (768, 768), 1.0, False), (2, (512, 512), 1.0, True)]
    rs, poses = [], flythrough_poses(len(views), 5150)
    for (vi, (wd, ht), srm, lit), (eye, at, up) in zip(views, poses):
        r = Renderer()
        r.RegisterDataset(vols[vi][3])
        r.Set2DTransFloat(tf)
        r.SetRendermode(1)
        r.SetUseLighting(lit)
        r.SetSampleRateModifier(srm)
        r.Resize(wd, ht)
        r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye, at=at, up=up)
        rs.append(r)
    Batch().Paint(rs)
    for k, ((vi, (wd, ht), srm, lit), (eye, at, up), r) in enumerate(zip(views, poses, rs)):
        w, _, raw, _ = vols[vi]
        stride = 4 if wd * ht > 600000 else 1
        ref, _, rc = O.render(raw, w.brick_size, w.overlap, tf, width=wd, height=ht, eye=eye,
                              at=at, up=up, srm=srm, mode=1, lighting=lit, want_counts=True,
                              row_stride=stride)
        rows = np.arange(0, ht, stride)
        img, cnt = r.ReadBackPixels(), r.ReadSampleCounts()
        check_rows(img, cnt, ref, rc, rows, f"batched 2D view {k}")
        assert (img[rows, :, 3] > 0).mean() > 0.01, k


def test_gpu_leaper_iso_1024_matches_oracle(cuda_ok):
    import torch
    w = ooc_lod(1024)
    d, raw = device_volume(torch, w)
    vol = gpu_volume(d, w)
    r = Renderer()
    r.RegisterDataset(vol)
    r.SetRendermode(2)
    r.SetIsoValue(w.extra["iso"])
    r.SetUseLighting(True)
    r.SetSampleRateModifier(w.srm)
    r.Resize(w.width, w.height)
    pool = Pool(vol, 4 << 30)
    for k, (eye, at, up) in enumerate(flythrough_poses(w.n_poses, w.seed + 77)[:300:150]):
        r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye, at=at, up=up)
        info = pool.Paint(r, max_passes=64)
        assert info.converged == 1, k
        one = pool.Paint(r, max_passes=1)
        assert one.passes == 1 and one.paged == 0
        page = pool.GetPageTable()
        img, cnt = r.ReadBackPixels(), r.ReadSampleCounts()
        ref, _, rc, missing = O.leaper_render(raw, w.brick_size, w.overlap,
                                              np.zeros((256, 4), np.float32), page,
                                              width=w.width, height=w.height, eye=eye, at=at,
                                              up=up, mode=2, lighting=True,
                                              isovalue=w.extra["iso"], srm=w.srm, row_stride=8)
        rows = np.arange(0, w.height, 8)
        check_rows(img, cnt, ref, rc, rows, f"GridLeaper iso 1024^3 pose {k}")
        assert (img[rows, :, 3] > 0).mean() > 0.05, k
        got = pool.GetRequests()
        # the sampled rows' requests are part of the whole frame's
        assert np.isin(missing, got).all(), k
