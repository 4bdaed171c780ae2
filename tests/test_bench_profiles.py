"""bench.py takes roofline traffic and issue figures from the committed ncu
summaries only for the kernel and capture mode they were measured on."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_profile_figures_by_kernel_and_capture_mode():
    sys.path.insert(0, ROOT)
    import bench
    wl = "plain 256MiB lambda=0.05 L=1024"
    kernel_of, traffic, issue = bench.profile_figures(wl, True)
    assert kernel_of["k_final"] == "k_copy<0>"
    # dram read + write of each kernel in the committed capture
    assert traffic == {"k_gwalk<1>": 303_178_240 + 328_277_760,
                       "k_wwalk<1>": 41_696_000 + 4_675_072,
                       "k_copy<0>": 370_545_920 + 224_338_432}
    assert set(issue) == {"k_gwalk<1>", "k_wwalk<1>", "k_copy<0>"}
    assert all(0 < v <= 100 for v in issue.values())
    # no uncaptured profile is committed: nothing is borrowed from the
    # capturing decode's kernels
    kernel_of, traffic, issue = bench.profile_figures(wl, False)
    assert kernel_of["k_final"] == "k_final<0>" and traffic == {} and issue == {}
    assert bench.profile_figures("plain 16MiB lambda=0.05 L=1024", True)[1:] == ({}, {})
