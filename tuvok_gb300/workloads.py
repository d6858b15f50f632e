"""Seeded synthetic workloads of the benchmark and the tests.

The reference publishes no benchmark data; every input here is generated from
a seed.  Configurations (all single-GPU):

* ``plain_small``  -- 256^3 uint8, 32 Gaussian blobs (centres uniform in the
  volume, sigma U[8, 40] voxels, peak U[64, 255]) + uniform integer noise in
  [-4, 4], clamped to 0..255; bricks of 64^3 core + 1 ghost voxel (Tuvok brick
  size 66, overlap 1); 256-entry float RGBA TF with a linear colour ramp and
  opacity 0 below 40 rising linearly to 0.6 at 255; 512x512, FOV 50 degrees,
  seeded orbit; sample-rate modifier 1.0; unlit.
* ``plain_large_lit`` -- 1024^3 uint16 holding 12-bit values: 256 blobs
  (sigma U[16, 80], peak U[512, 3584]) + 3-octave value noise of amplitude
  409.5 (10% of range, base cell 128 voxels), clamped to 0..4095; bricks of
  128^3 core + 1 ghost voxel; 4096-entry TF with two opaque bands (alpha 0
  elsewhere, so most bricks are empty); Blinn-Phong lighting (ka 0.2, kd 0.6,
  ks 0.2, shininess 32); 1920x1080; sample-rate modifier 1.5; 120 seeded poses.

Sample-rate modifier semantics are the reference's (GLRaycaster.cpp:255): the
step is 0.5/srm voxel, so srm 1.0 takes 2 samples per voxel.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Workload:
    name: str
    dims: tuple            # (x, y, z)
    dtype: type
    vmax: float
    n_blobs: int
    sigma: tuple
    peak: tuple
    noise_amp: float
    noise_octaves: int
    noise_cell: float
    int_noise: bool
    brick_core: int
    overlap: int
    width: int
    height: int
    srm: float
    lighting: bool
    light_model: int       # 0 reference, 1 Blinn-Phong
    tf_kind: str
    seed: int
    n_poses: int = 120
    extra: dict = field(default_factory=dict)

    @property
    def brick_size(self):
        c = self.brick_core + 2 * self.overlap
        return (c, c, c)

    def blobs(self) -> np.ndarray:
        rng = np.random.default_rng(self.seed)
        n = self.n_blobs
        t = np.zeros((n, 7), dtype=np.float32)
        for a in range(3):
            t[:, a] = rng.uniform(0, self.dims[a], n)
        t[:, 3] = rng.uniform(*self.sigma, n)
        t[:, 4] = rng.uniform(*self.peak, n)
        return t

    def tf(self) -> np.ndarray:
        return make_tf(self.tf_kind)

    def poses(self, n=None, seed_offset=0):
        return orbit_poses(n or self.n_poses, self.seed + 1000 + seed_offset)


def make_tf(kind: str) -> np.ndarray:
    if kind == "ramp256":
        i = np.arange(256, dtype=np.float64)
        t = np.zeros((256, 4), dtype=np.float32)
        t[:, 0] = i / 255.0
        t[:, 1] = 0.8 * i / 255.0
        t[:, 2] = 1.0 - i / 255.0
        t[:, 3] = np.where(i < 40, 0.0, 0.6 * (i - 40) / (255 - 40))
        return t
    if kind == "bands4096":
        i = np.arange(4096, dtype=np.float64)
        t = np.zeros((4096, 4), dtype=np.float32)
        for centre, colour in ((1400.0, (1.0, 0.62, 0.25)), (2600.0, (0.35, 0.65, 1.0))):
            d = np.abs(i - centre)
            a = np.clip((80.0 - d) / 30.0, 0.0, 1.0) * 0.9
            m = a > 0
            t[m, 0], t[m, 1], t[m, 2] = colour
            t[:, 3] = np.maximum(t[:, 3], a)
        return t
    raise ValueError(kind)


def orbit_poses(n: int, seed: int, radius: float = 1.6):
    """Seeded orbit: eye on a sphere of `radius` around the origin, looking at it."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        az = rng.uniform(0, 2 * math.pi)
        el = rng.uniform(-math.radians(60), math.radians(60))
        eye = (radius * math.cos(el) * math.sin(az), radius * math.sin(el),
               radius * math.cos(el) * math.cos(az))
        out.append((eye, (0.0, 0.0, 0.0), (0.0, 1.0, 0.0)))
    return out


PLAIN_SMALL = Workload(
    name="plain_small", dims=(256, 256, 256), dtype=np.uint8, vmax=255, n_blobs=32,
    sigma=(8, 40), peak=(64, 255), noise_amp=4, noise_octaves=0, noise_cell=0, int_noise=True,
    brick_core=64, overlap=1, width=512, height=512, srm=1.0, lighting=False, light_model=0,
    tf_kind="ramp256", seed=1234)

PLAIN_LARGE_LIT = Workload(
    name="plain_large_lit", dims=(1024, 1024, 1024), dtype=np.uint16, vmax=4095, n_blobs=256,
    sigma=(16, 80), peak=(512, 3584), noise_amp=409.5, noise_octaves=3, noise_cell=128.0,
    int_noise=False, brick_core=128, overlap=1, width=1920, height=1080, srm=1.5,
    lighting=True, light_model=1, tf_kind="bands4096", seed=4321)

# The large lit scene at half resolution (512^3, blobs and noise cells scaled
# by 1/2): the profiling case whose brick pool (~280 MB) still exceeds L2.
PLAIN_MEDIUM_LIT = Workload(
    name="plain_medium_lit", dims=(512, 512, 512), dtype=np.uint16, vmax=4095, n_blobs=256,
    sigma=(8, 40), peak=(512, 3584), noise_amp=409.5, noise_octaves=3, noise_cell=64.0,
    int_noise=False, brick_core=128, overlap=1, width=1920, height=1080, srm=1.5,
    lighting=True, light_model=1, tf_kind="bands4096", seed=4321)

WORKLOADS = {w.name: w for w in (PLAIN_SMALL, PLAIN_LARGE_LIT, PLAIN_MEDIUM_LIT)}


# Out-of-core LOD rendering (GridLeaper): a logical N^3 uint8 volume of 1024
# blobs (sigma and noise cell scaled with N / 4096) + 4-octave value noise of
# amplitude 25.5 (10% of range); bricks of 128^3 core + 1 ghost voxel with
# every coarser LOD down to one brick; isosurface 128, lit, 1920x1080, 300
# seeded fly-through frames; a brick cache of (N / 4096)^3 * 24 GB paged from
# pinned host memory.
def ooc_lod(n=2048):
    f = n / 4096.0
    return Workload(
        name=f"ooc_lod_iso_{n}", dims=(n, n, n), dtype=np.uint8, vmax=255, n_blobs=1024,
        sigma=(32 * f, 160 * f), peak=(96, 255), noise_amp=25.5, noise_octaves=4,
        noise_cell=256.0 * f, int_noise=False, brick_core=128, overlap=1, width=1920,
        height=1080, srm=1.0, lighting=True, light_model=0, tf_kind="", seed=4096, n_poses=300,
        extra={"iso": 128.0, "cache_bytes": int(24e9 * f ** 3)})


def flythrough_poses(n: int, seed: int):
    """Seeded fly-through around and into the unit volume: the eye follows a
    smooth closed curve (distance 0.55..1.45 from the centre, elevation within
    +-35 degrees) and looks at a point that wanders near the centre; the
    camera moves a little each frame, as in an interactive session."""
    rng = np.random.default_rng(seed)
    ph = rng.uniform(0, 2 * math.pi, 6)
    out = []
    for i in range(n):
        t = i / n
        az = 2 * math.pi * t + ph[0]
        r = 1.0 + 0.45 * math.sin(2 * math.pi * 2 * t + ph[1])
        el = math.radians(35) * math.sin(2 * math.pi * 3 * t + ph[2])
        eye = (r * math.cos(el) * math.sin(az), r * math.sin(el), r * math.cos(el) * math.cos(az))
        at = (0.15 * math.sin(2 * math.pi * 5 * t + ph[3]),
              0.15 * math.sin(2 * math.pi * 4 * t + ph[4]),
              0.15 * math.sin(2 * math.pi * 3 * t + ph[5]))
        out.append((eye, at, (0.0, 1.0, 0.0)))
    return out


# Batching: 64 views of mixed sizes over four volumes made with the plain_small
# blob rules (values scaled to the type's range), a 256x256 float 2D TF of
# three Gaussian lobes over (value, |gradient| * gradient scale), sample-rate
# modifier in {0.5, 1, 2}, lit and unlit mixed; bricks 64^3 core + 1 ghost.
BATCH_VOLUMES = [
    Workload(name="batch_a", dims=(128, 128, 128), dtype=np.uint8, vmax=255, n_blobs=32,
             sigma=(4, 20), peak=(64, 255), noise_amp=4, noise_octaves=0, noise_cell=0,
             int_noise=True, brick_core=64, overlap=1, width=0, height=0, srm=1.0,
             lighting=False, light_model=0, tf_kind="", seed=501),
    Workload(name="batch_b", dims=(256, 256, 256), dtype=np.uint16, vmax=4095, n_blobs=32,
             sigma=(8, 40), peak=(1024, 4095), noise_amp=64, noise_octaves=0, noise_cell=0,
             int_noise=True, brick_core=64, overlap=1, width=0, height=0, srm=1.0,
             lighting=False, light_model=0, tf_kind="", seed=502),
    Workload(name="batch_c", dims=(384, 384, 256), dtype=np.uint8, vmax=255, n_blobs=32,
             sigma=(10, 50), peak=(64, 255), noise_amp=4, noise_octaves=0, noise_cell=0,
             int_noise=True, brick_core=64, overlap=1, width=0, height=0, srm=1.0,
             lighting=False, light_model=0, tf_kind="", seed=503),
    Workload(name="batch_d", dims=(512, 512, 512), dtype=np.uint16, vmax=4095, n_blobs=32,
             sigma=(16, 80), peak=(1024, 4095), noise_amp=64, noise_octaves=0, noise_cell=0,
             int_noise=True, brick_core=64, overlap=1, width=0, height=0, srm=1.0,
             lighting=False, light_model=0, tf_kind="", seed=504),
]
BATCH_SIZES = [(256, 256), (512, 512), (768, 768), (1024, 1024), (1280, 720)]


def tf2d_lobes(w=256, h=256, seed=77):
    """2D TF of three Gaussian lobes (RGBA float, [h][w]; x = value, y = gradient)."""
    rng = np.random.default_rng(seed)
    v, g = np.meshgrid(np.linspace(0, 1, w), np.linspace(0, 1, h))
    t = np.zeros((h, w, 4), dtype=np.float32)
    for _ in range(3):
        cv, cg, sv, sg = (rng.uniform(0.3, 0.9), rng.uniform(0.0, 0.6), rng.uniform(0.04, 0.12),
                          rng.uniform(0.1, 0.3))
        a = np.exp(-((v - cv) ** 2 / (2 * sv * sv) + (g - cg) ** 2 / (2 * sg * sg)))
        col = rng.uniform(0.2, 1.0, 3)
        for c in range(3):
            t[..., c] = np.maximum(t[..., c], (a * col[c]).astype(np.float32))
        t[..., 3] = np.maximum(t[..., 3], (0.6 * a).astype(np.float32))
    t[..., 3] = np.where(t[..., 3] < 0.02, 0.0, t[..., 3])
    return t


# Many small views (thumbnails, multi-view displays): where one launch for all
# of them matters most.
SMALL_BATCH_SIZES = [(96, 96), (128, 128), (160, 120), (192, 192), (256, 256)]


def batch_views(n=64, seed=900, sizes=None):
    """(volume index, (width, height), srm, lit) per view, seeded."""
    sizes = sizes or BATCH_SIZES
    rng = np.random.default_rng(seed)
    return [(int(rng.integers(0, len(BATCH_VOLUMES))),
             sizes[int(rng.integers(0, len(sizes)))],
             float(rng.choice([0.5, 1.0, 2.0])), bool(rng.integers(0, 2))) for _ in range(n)]


def numpy_blob_volume(dims, dtype, n_blobs, sigma, peak, vmax, seed, noise=0):
    """Small CPU-made volume for tests (input creation only): [z, y, x] array."""
    rng = np.random.default_rng(seed)
    x, y, z = dims
    zz, yy, xx = np.meshgrid(np.arange(z), np.arange(y), np.arange(x), indexing="ij")
    v = np.zeros((z, y, x), dtype=np.float64)
    for _ in range(n_blobs):
        c = rng.uniform(0, 1, 3) * np.array(dims)
        s = rng.uniform(*sigma)
        p = rng.uniform(*peak)
        d2 = (xx - c[0]) ** 2 + (yy - c[1]) ** 2 + (zz - c[2]) ** 2
        v += p * np.exp(-d2 / (2 * s * s))
    if noise:
        v += rng.integers(-noise, noise + 1, size=v.shape)
    return np.clip(np.floor(v + 0.5), 0, vmax).astype(dtype)
