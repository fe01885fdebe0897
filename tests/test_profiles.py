"""The committed ncu summary of the C2 frame carries, for every kernel ncu captured in full (the
splat, push level 0, the gathering and the one-block pyramid of the host-buffer frame), the
per-launch DRAM bytes and issue-slot use that bench.py reports beside the roofline fraction, and
bench.py reads them back."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402

KERNELS = ["ism_splat", "push0", "final_gather", "pyramid"]


@pytest.mark.parametrize("kernel", KERNELS)
def test_summary_has_traffic_and_issue(kernel):
    traffic = bench.ncu_traffic(kernel)
    issue = bench.ncu_traffic(kernel, "issue")
    assert traffic is not None and 1e6 < traffic < 1e9, traffic
    assert issue is not None and 0.0 < issue <= 100.0, issue


def test_unknown_kernel_reads_none():
    assert bench.ncu_traffic("no_such_kernel") is None
    assert bench.ncu_traffic("no_such_kernel", "issue") is None


def test_other_workload_reads_none():
    """Figures of the 1080p capture are not reported for another workload."""
    assert bench.ncu_traffic("final_gather", workload="c1_640x360_n256") is None
