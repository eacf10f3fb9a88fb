"""The kernels' cos(theta)-indexed directivity table (dir_ctable.inc, used by directivity2_ctab)
is the one dir_ctable.py derives, follows the reference's T4010A1 directivity
(t4010a1.rs:18-71,107-120) on every interval side to float32 rounding, and puts each bin edge
(the exact float thresholds of bin_edges.py) in the interval the kernels' index arithmetic
gives for it."""
import os
import re
import sys

import numpy as np

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                    "acoustic-field-calculator_gb300", "csrc")
sys.path.insert(0, CSRC)
import bin_edges as BE  # noqa: E402
import dir_ctable as CT  # noqa: E402


def _parse(name):
    text = open(os.path.join(CSRC, "dir_ctable.inc")).read()
    block = text[text.index(f"#define {name}"):]
    block = block[block.index("{") + 1:]
    end = block.index("\n}")
    vals = re.findall(r"-?0x[0-9a-fA-F.]+p[-+]?\d+f|-?\d+\.\d+f", block[:end])
    return np.array([float.fromhex(v.rstrip("f")) if "x" in v else float(v.rstrip("f"))
                     for v in vals], dtype=np.float32)


def test_header_is_the_derived_table():
    ne, cf, _ = CT.table()
    np.testing.assert_array_equal(_parse("AFC_CTAB_NEGEDGE_INIT"), ne)
    np.testing.assert_array_equal(_parse("AFC_CTAB_COEF_INIT").reshape(-1, 4), cf)


def test_cubics_follow_the_directivity_on_every_side():
    ne, cf, bins = CT.table()
    assert CT.check(ne, cf, bins) <= 2e-7


def test_edges_sit_in_the_interval_the_kernel_indexes():
    ne, _, bins = CT.table()
    ths = BE.thresholds()
    for b in range(3, 11):
        e = np.float32(ths[b - 1])
        # the kernels' index: RD(c K + 2^23 + BIAS) & (SIZE - 1)
        i = (int(np.floor(np.float64(e) * CT.K)) + CT.BIAS) & (CT.SIZE - 1)
        assert ne[i] == -e
        assert bins[2 * i] == b - 1 and bins[2 * i + 1] == b
    # and the back axis: the two intervals that meet at c = -1
    for c in (np.float32(-1.0), np.nextafter(np.float32(-1.0), np.float32(-2.0))):
        i = (int(np.floor(np.float64(c) * CT.K)) + CT.BIAS) & (CT.SIZE - 1)
        assert ne[i] == np.float32(1.0)
    assert np.count_nonzero(ne != np.float32(-CT.NO_EDGE)) == 10
