"""TF scaling methods (AbstrRenderer::SetScalingMethod): with
SMETH_BIAS_AND_SCALE the 1D coordinate is value * (|min| + |max|) of the data
range, as GLRaycaster's shaders compute it (GLRaycaster.cpp:577-584; the bias
uniform is never selected).  Against the oracle with the usual tolerance; 2D
and iso modes do not change."""
import numpy as np
import pytest

import oracle as O
from test_gpu_lod_render import make, vols  # noqa: F401  (fixture)
from test_gpu_render import compare, tf2d

pytestmark = pytest.mark.gpu


def band_tf(n):
    """Alpha only near the top of the table: the scaled coordinate lands there."""
    t = np.zeros((n, 4), dtype=np.float32)
    i = np.arange(n) / (n - 1)
    t[:, 0], t[:, 1], t[:, 2] = i, 1 - i, 0.5
    t[:, 3] = np.where(i > 0.6, 0.05 + 0.3 * i, 0.0)
    return t


@pytest.mark.parametrize("vk,lit", [("u8", False), ("u8", True), ("u16", False),
                                    ("u16", True)])
def test_gpu_bias_and_scale_matches_oracle(cuda_ok, vols, vk, lit):  # noqa: F811
    raw = vols[vk]
    tf = band_tf(256 if vk == "u8" else 1024)
    vol, r = make(raw, 18, 1, tf, 0, lit)
    eye = (0.4, 0.3, 1.4)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye)
    r.Resize(72, 64)
    r.Paint()
    bit_width = r.ReadBackPixels().copy()
    r.SetScalingMethod(r.SMETH_BIAS_AND_SCALE)
    r.Paint()
    img, cnt = r.ReadBackPixels(), r.ReadSampleCounts()
    ref, n, rc = O.render(raw, (18,) * 3, 1, tf, width=72, height=64, eye=eye, mode=0,
                          lighting=lit, want_counts=True, bias_scale=True)
    compare(img, ref, f"{vk} lit={lit}")
    np.testing.assert_array_equal(cnt, rc)
    assert not np.array_equal(img, bit_width)
    r.SetScalingMethod(r.SMETH_BIT_WIDTH)
    r.Paint()
    np.testing.assert_array_equal(r.ReadBackPixels(), bit_width)


def test_gpu_bias_and_scale_leaves_2d_alone(cuda_ok, vols):  # noqa: F811
    raw = vols["u8"]
    vol, r = make(raw, 18, 1, tf2d(), 1, True)
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=(0.4, 0.3, 1.4))
    r.Resize(72, 64)
    r.Paint()
    a = r.ReadBackPixels().copy()
    r.SetScalingMethod(r.SMETH_BIAS_AND_SCALE)
    r.Paint()
    np.testing.assert_array_equal(r.ReadBackPixels(), a)
