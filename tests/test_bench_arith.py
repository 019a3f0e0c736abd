"""The bench's arithmetic on the CPU: the launch count of the timed steps, the
step's lower bound, and the force pass's issue fraction recomputed from the
fields a bench line carries."""
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_launch_count_of_the_timed_steps():
    # 20 kept-list steps from step counter 2571: no drift removal (no multiple
    # of 100 in 2571..2590), 7 rebuilds, one loop launch, no reorder
    k = bench.gpu_launches(20, True, 7, 2571, 0)
    assert k == 20 * bench.KERNELS_PER_KEPT_STEP + 7 * bench.KERNELS_PER_REBUILD + 1
    # across step 2600: the drift removal once, and a reorder splitting the loop
    k2 = bench.gpu_launches(20, True, 7, 2590, 1)
    assert k2 == (20 * bench.KERNELS_PER_KEPT_STEP + 7 * bench.KERNELS_PER_REBUILD
                  + bench.KERNELS_PER_CM + 2 + bench.KERNELS_PER_REORDER)
    # without kept lists every step runs every kernel and there are no rebuild bodies
    assert bench.gpu_launches(10, False, 0, 1, 0) == 10 * bench.KERNELS_PER_STEP + 1


def test_step_lower_bound(monkeypatch):
    monkeypatch.setattr(bench, "measured_peaks", lambda: (7000.0, "measured"))
    pairs, n = 150_000_000, 1_000_000
    peak = 4 * 32 * 152 * 2070e6 / 1e12
    r = bench.step_roofline({"ordered_pairs": pairs, "peak": peak}, n, 2.2)
    want = {"force_ms": bench.OPS_PER_ORDERED_PAIR["force"] * pairs / (peak * 1e12) * 1e3,
            "density_ms": bench.OPS_PER_ORDERED_PAIR["density"] * pairs / (peak * 1e12) * 1e3,
            "hbm_ms": bench.STEP_BYTES_PER_PARTICLE * n / 7000e9 * 1e3}
    for key, v in want.items():
        assert r["parts"][key] == pytest.approx(v, rel=1e-12)
    assert r["frac"] == pytest.approx(sum(want.values()) / 2.2, rel=1e-12)


def test_issue_fraction_from_a_bench_line():
    # fields of a recorded membrane_1m line (984,040 beads, 152 SMs at 2,070 MHz)
    line = {"kernel_ms": 1.1676479578018188, "ordered_pairs": 152733500,
            "ops_per_ordered_pair": 134, "peak": 40.27392, "frac": 0.43521441882517997}
    achieved = line["ops_per_ordered_pair"] * line["ordered_pairs"] / (line["kernel_ms"] * 1e-3) / 1e12
    assert 4 * 32 * 152 * 2070e6 / 1e12 == pytest.approx(line["peak"], rel=1e-12)
    assert achieved / line["peak"] == pytest.approx(line["frac"], rel=1e-12)
    assert bench.OPS_PER_ORDERED_PAIR["force"] == line["ops_per_ordered_pair"]
