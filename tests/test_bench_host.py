"""Host-side logic of bench.py (no GPU): the roofline object built from per-launch
kernel times, the kernel names of batched launch groups, and the committed DRAM traffic
ratios it reads."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_kernel_names_of_batched_groups():
    assert bench.kernel_of("batched 23x f32 tc3xtf32 axis1: mat diagnd") == "angular_tc_kernel_batched"
    assert bench.kernel_of("batched 5x f32 tcbf16x3 parity axis1: mat") == "angular_tc_kernel_batched"
    assert bench.kernel_of("batched 9x f32 sweep fftpair axis0: fft diag1d fft diagnd") == "fft_pair_kernel_batched"
    assert bench.kernel_of("batched 9x f64 sweep axis0: fft diag1d fft diagnd") == "pass_kernel_batched"
    assert bench.kernel_of("batched 9x ff sweep fftpair axis0: fft diag1d fft diagnd") == "fft_pair_kernel_batched_ff"
    assert bench.kernel_of("batched 9x ff sweep axis1: mat diagnd norm") == "pass_kernel_batched"


def test_roofline_aggregates_all_launches_of_the_dominant_kernel():
    times = [("batched 2x f32 tc3xtf32 axis1: a", 2, 3.0, 6e9),
             ("batched 3x f32 tc3xtf32 axis1: b", 1, 1.0, 2e9),
             ("batched 4x f32 sweep fftpair axis0: c", 4, 2.0, 4e9)]
    r = bench.roofline_from(times, 6.0)
    assert r["kernel"] == "angular_tc_kernel_batched"
    assert r["launches"] == 3 and r["groups"] == 2
    # 8e9 algorithmic bytes over 4 ms of launches
    assert r["achieved"] == pytest.approx(8e9 / 4e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert r["share_of_timed"] == pytest.approx(4.0 / 6.0)
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"
    ratio = bench.ncu_traffic().get("angular_tc_kernel_batched")
    if ratio is not None:
        assert r["traffic"] == pytest.approx(ratio * 8e9 / 3)


def test_committed_traffic_ratios_parse():
    t = bench.ncu_traffic()
    assert set(t) >= {"angular_tc_kernel_batched", "fft_pair_kernel_batched"}
    assert all(0.5 < v < 1.5 for v in t.values())


def test_no_times_no_roofline():
    assert bench.roofline_from([], 1.0) is None
