"""The bench's second roofline of the pair enumeration: warp instructions per second against
the issue peak (one warp instruction per clock on each of the 4 x 152 SM sub-partitions),
from the instruction count ncu measured for the same shapes.  Host arithmetic only."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_issue_roofline_of_the_measured_shapes():
    r = bench.pair_issue_roofline("bcc64", 0.0045, 1216, 0.32, 2070.0)
    inst = bench.PAIR_WARP_INSTRUCTIONS[("bcc64", 0.0045, 1216)]
    assert r["bound"] == "issue" and r["warp_instructions_per_launch"] == inst
    assert abs(r["achieved"] - inst / 0.32e-3 / 1e9) < 1e-9 * r["achieved"]
    assert abs(r["peak"] - 4 * 152 * 2.07) < 1e-9  # G warp-instructions/s at 2070 MHz
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-12
    assert 0 < r["frac"] < 1


def test_issue_roofline_needs_a_measured_count_and_a_clock():
    assert bench.pair_issue_roofline("bcc64", 0.005, 1216, 0.32, 2070.0) is None  # another cell
    assert bench.pair_issue_roofline("bcc64", 0.0045, 608, 0.32, 2070.0) is None  # another grid
    assert bench.pair_issue_roofline("bcc32", 0.0045, 1216, 0.32, 2070.0) is None  # another specimen
    assert bench.pair_issue_roofline("bcc64", 0.0045, 1216, 0.32, None) is None  # no clock sample
