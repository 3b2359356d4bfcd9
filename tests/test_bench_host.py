"""Host-side helpers of bench.py (no GPU): sysfs cpulist parsing for the
GPU-local pinning of the end-to-end step's host buffers."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import bench  # noqa: E402


def test_parse_cpulist():
    assert bench.parse_cpulist("0-3,8,10-11\n") == {0, 1, 2, 3, 8, 10, 11}
    assert bench.parse_cpulist("5") == {5}
    assert bench.parse_cpulist("0-15") == set(range(16))
    assert bench.parse_cpulist("") == set()
