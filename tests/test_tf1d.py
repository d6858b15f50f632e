"""TransferFunction1D (IO/TransferFunction1D.cpp) as tuvok_gb300's table
functions (tvk_tf1d_*, host code in libtvk.so, no GPU needed) against the
reference's own class: the golden vectors tests/golden/tf1d/make_tf1d_golden.py
wrote from it, and the live class where oracle/_ref is built.  Tables, non-zero
limits and byte arrays are compared bit for bit (NaN where the reference
divides by zero)."""
from pathlib import Path

import numpy as np
import pytest

import refconv
from tuvok_gb300 import TransferFunction1D

GOLDEN = np.load(Path(__file__).resolve().parent / "golden" / "tf1d" / "tf1d.npz")


def _cases(prefix):
    return sorted({int(k[len(prefix):].split("_")[0]) for k in GOLDEN.files
                   if k.startswith(prefix) and k[len(prefix)].isdigit()})


def _same(a, b, what):
    a = np.asarray(a, dtype=np.float32)
    b = np.asarray(b, dtype=np.float32)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32)) or \
        np.array_equal(a, b, equal_nan=True), f"{what}: tables differ"


def _tf(table):
    tf = TransferFunction1D(table.shape[0])
    tf.GetColorData()[:] = table
    return tf


def test_set_std_function_matches_reference():
    for i in _cases("std"):
        t = GOLDEN[f"std{i}_in"]
        c, g, comp, inv = GOLDEN[f"std{i}_args"]
        tf = _tf(t)
        if int(comp) < 0:
            tf.SetStdFunction(float(c), float(g))
        else:
            tf.SetStdFunction(float(c), float(g), int(comp), bool(inv))
        _same(tf.GetColorData(), GOLDEN[f"std{i}_out"], f"std case {i} ({c}, {g}, {comp}, {inv})")
        assert tf.GetNonZeroLimits() == tuple(int(x) for x in GOLDEN[f"std{i}_lim"]), i


def test_set_bytes_matches_reference():
    for i in _cases("set"):
        tf = TransferFunction1D()
        tf.Set(GOLDEN[f"set{i}_in"])
        _same(tf.GetColorData(), GOLDEN[f"set{i}_out"], f"set case {i}")
        assert tf.GetNonZeroLimits() == tuple(int(x) for x in GOLDEN[f"set{i}_lim"]), i


def test_resample_and_fill_or_truncate_match_reference():
    for i in _cases("res"):
        t = GOLDEN[f"res{i}_in"]
        target = GOLDEN[f"res{i}_out"].shape[0]
        tf = _tf(t)
        tf.Resample(target)
        _same(tf.GetColorData(), GOLDEN[f"res{i}_out"], f"resample case {i} ({t.shape[0]}->{target})")
        assert tf.GetNonZeroLimits() == tuple(int(x) for x in GOLDEN[f"res{i}_lim"]), i
        tf = _tf(t)
        tf.FillOrTruncate(target)
        _same(tf.GetColorData(), GOLDEN[f"fot{i}_out"], f"fill/truncate case {i}")


def test_byte_array_matches_reference():
    for i in _cases("bytes"):
        tf = _tf(GOLDEN[f"bytes{i}_in"])
        r = int(GOLDEN[f"bytes{i}_range"][0])
        np.testing.assert_array_equal(tf.GetByteArray(r), GOLDEN[f"bytes{i}_out"])


def test_nonzero_limits_edge_cases():
    tf = TransferFunction1D(16)
    tf.ComputeNonZeroLimits()
    assert tf.GetNonZeroLimits() == (16, 0)  # no opaque entry
    tf.GetColorData()[5, 3] = 0.5
    tf.ComputeNonZeroLimits()
    assert tf.GetNonZeroLimits() == (5, 5)
    tf.Clear()
    assert tf.GetNonZeroLimits() == (0, 0) and not tf.GetColorData().any()


def test_save_load_round_trip(tmp_path):
    rng = np.random.default_rng(5)
    tf = _tf(rng.uniform(0, 1, (37, 4)).astype(np.float32))
    p = tmp_path / "a.1dt"
    tf.Save(p)
    back = TransferFunction1D.FromFile(p)
    # the text format keeps 6 significant digits (iostream default)
    np.testing.assert_allclose(back.GetColorData(), tf.GetColorData(), rtol=1e-5, atol=1e-6)
    back2 = TransferFunction1D.FromFile(p, 100)
    assert back2.GetSize() == 100
    # a truncated file fails as Load(istream) fails
    text = p.read_text().split()
    (tmp_path / "b.1dt").write_text(" ".join(text[:-3]))
    with pytest.raises(Exception):
        TransferFunction1D.FromFile(tmp_path / "b.1dt")


@pytest.mark.skipif(not refconv.available(), reason="reference class not built here")
def test_live_reference_and_file_format(tmp_path):
    """The live class on fresh inputs, and files written by either side read
    by the other with identical text."""
    rng = np.random.default_rng(99)
    for n in (3, 64, 4096):
        t = rng.uniform(-0.3, 1.3, (n, 4)).astype(np.float32)
        for c, g in ((0.4, 0.3), (0.9, 0.05)):
            ref, lim = refconv.tf1d_std(t, c, g, 1, True)
            tf = _tf(t)
            tf.SetStdFunction(c, g, 1, True)
            _same(tf.GetColorData(), ref, f"live std {n}")
            assert tf.GetNonZeroLimits() == lim
        for target in (5, 333, 5000):
            ref, lim = refconv.tf1d_resample(t, target)
            tf = _tf(t)
            tf.Resample(target)
            _same(tf.GetColorData(), ref, f"live resample {n}->{target}")
        a, b = tmp_path / "ours.1dt", tmp_path / "ref.1dt"
        _tf(t).Save(a)
        assert refconv.tf1d_save(t, b)
        assert a.read_text() == b.read_text()
        loaded, ok = refconv.tf1d_load(a)
        assert ok
        _same(TransferFunction1D.FromFile(b).GetColorData(), loaded, "load")
