"""The kernels' directivity table (AFC_DIR_TABLE_INIT in propagate.cuh, the reference's cubics
re-expanded about each bin's centre) is the derived one and reproduces the oracle's T4010A1
directivity (t4010a1.rs:107-120) inside every bin."""
import os
import re
import sys

import numpy as np

import oracle as O

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                    "acoustic-field-calculator_gb300", "csrc")
sys.path.insert(0, CSRC)
import dir_table as DT  # noqa: E402


def _header_table():
    text = open(os.path.join(CSRC, "propagate.cuh")).read()
    block = text[text.index("#define AFC_DIR_TABLE_INIT"):]
    block = block[:block.index("constexpr")]
    rows = re.findall(r"\{([^{}]*)\}", block)
    vals = [[float.fromhex(v.strip().rstrip("f")) if "x" in v else float(v.strip().rstrip("f"))
             for v in r.split(",")] for r in rows]
    return np.array(vals, dtype=np.float32)


def test_header_table_is_the_derived_one():
    t = _header_table()
    assert t.shape == (32, 4)
    np.testing.assert_array_equal(t, DT.table())


def test_centred_cubics_follow_the_oracle_inside_every_bin():
    t = DT.table()
    div = DT.ANGLE_DIV
    worst = 0.0
    for i in range(1, 10):
        # interior of bin i: theta in ((i - 1) div, i div), away from the edges
        th = np.linspace((i - 1) * float(div) + 1e-4, i * float(div) - 1e-4, 2001).astype(np.float32)
        ref = np.array([O.directivity(float(x)) for x in th])
        xc = (th - (np.float32(i) - np.float32(0.5)) * div).astype(np.float32)
        A, B, C, D = t[i]
        got = (A + (B + (C + D * xc) * xc) * xc).astype(np.float32)
        worst = max(worst, float(np.max(np.abs(got - ref))))
    assert worst < 5e-7, worst
    assert DT.check(t) < 1e-7
    # beyond 90 degrees, and the wrapped entry for theta just below 0
    assert np.all(t[10:31] == 0) and tuple(t[31]) == (1, 0, 0, 0) and tuple(t[0]) == (1, 0, 0, 0)
