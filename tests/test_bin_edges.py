"""The exact directivity-bin thresholds of the field kernels (kBinCos1..10 in propagate.cuh)
reproduce the reference's bin ceil(acosf(c) / ANGLE_DIV) for every float c around each edge,
with acosf the platform libm's (glibc's, which Rust's f32::acos calls; the oracle's default
mode).  Run on the GPU machine too, this also checks that its libm agrees with the one the
thresholds were derived with."""
import os
import re
import sys

import numpy as np

import oracle as O

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                    "acoustic-field-calculator_gb300", "csrc")
sys.path.insert(0, CSRC)
import bin_edges as BE  # noqa: E402


def _header_thresholds():
    text = open(os.path.join(CSRC, "propagate.cuh")).read()
    vals = {int(b): float.fromhex(h) for b, h in
            re.findall(r"constexpr float kBinCos(\d+) = ([-0-9a-fx.p+]+)f;", text)}
    assert sorted(vals) == list(range(1, 11))
    return [np.float32(vals[b]) for b in range(1, 11)]


def test_header_thresholds_are_the_derived_ones():
    assert [float(t) for t in _header_thresholds()] == [float(t) for t in BE.thresholds()]


def test_thresholds_reproduce_the_oracle_bins_around_every_edge():
    ths = _header_thresholds()
    lo_key = int(BE._f32_to_key(np.float32(-1.0)))
    hi_key = int(BE._f32_to_key(np.float32(1.0)))
    keys = np.concatenate([np.arange(max(lo_key, int(BE._f32_to_key(t)) - 20000),
                                     min(hi_key, int(BE._f32_to_key(t)) + 20000) + 1)
                           for t in ths])
    c = BE._key_to_f32(keys)
    rng = np.random.default_rng(1)
    c = np.concatenate([c, rng.uniform(-1, 1, 200000).astype(np.float32),
                        np.float32([1.0, -1.0, 0.0, -0.0, np.nan])])
    ref = O.bins_of_cos(c)
    assert np.array_equal(BE.bin_from_thresholds(c, ths), ref)
