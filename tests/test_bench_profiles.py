"""bench.py takes roofline traffic and issue figures from the committed ncu
summaries only for the kernel and capture mode they were measured on."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_profile_figures_by_kernel_and_capture_mode():
    sys.path.insert(0, ROOT)
    import bench
    wl = "plain 256MiB lambda=0.05 L=1024"
    kernel_of, traffic, issue, inst = bench.profile_figures(wl, True)
    assert kernel_of["k_final"] == "k_copy<0>"
    # dram read + write of each kernel in the committed captures
    assert traffic == {"k_gwalk<1>": 631_123_968, "k_wwalk<1>": 46_963_712,
                       "k_copy<0>": 594_449_920}
    assert set(issue) == set(inst) == {"k_gwalk<1>", "k_wwalk<1>", "k_copy<0>"}
    assert all(0 < v <= 100 for v in issue.values())
    # thread instructions per output symbol of the G pass (268 M symbols)
    assert 30 < inst["k_gwalk<1>"] / 268_435_456 < 40
    # no uncaptured profile is committed: nothing is borrowed from the
    # capturing decode's kernels
    kernel_of, traffic, issue, inst = bench.profile_figures(wl, False)
    assert kernel_of["k_final"] == "k_final<0>" and traffic == {} and issue == {} and inst == {}
    assert bench.profile_figures("plain 16MiB lambda=0.05 L=1024", True)[1:] == ({}, {}, {})
