"""The device count of ordered pairs within the cutoff (idpd_pair_count):
the n_p x N of the pair passes' roofline, counted by the density pass. It
must equal a brute-force count of the pairs with minimum-image distance
r < 1 (i != j) on the same positions, in the FP32 engine (cell sweep and
kept lists) and in the plain FP64 arm."""
import numpy as np
import pytest

from helpers import mdpd_params, mixed_system
from implicit_dpd_gb300.abi import CFG_FP64_PAIRS
from implicit_dpd_gb300.engine import Engine

pytestmark = pytest.mark.gpu


def brute_pairs(pos, box):
    n = len(pos)
    total = 0
    for i0 in range(0, n, 512):
        d = pos[i0:i0 + 512, None, :] - pos[None, :, :]
        d -= box * np.round(d / box)
        r2 = (d ** 2).sum(-1)
        r2[np.arange(min(512, n - i0)), np.arange(i0, min(i0 + 512, n))] = 2.0
        total += int((r2 < 1.0).sum())
    return total


@pytest.mark.parametrize("flags", [0, CFG_FP64_PAIRS])
def test_pair_count_equals_brute_force(flags):
    box, st, _ = mixed_system()
    e = Engine(flags=flags)
    e.set_params(mdpd_params(box))
    e.upload(st)
    assert e.pair_count() == 0  # no density pass yet
    e.density()
    assert e.pair_count() == brute_pairs(st["pos"], box)
    e.close()


def test_pair_count_with_kept_lists_follows_the_steps():
    box, st, n_amp = mixed_system(seed=3)
    e = Engine()
    e.set_params(mdpd_params(box))
    e.upload(st)
    e.build_topology(n_amp)
    e.set_tuning(1, 0.2)
    for _ in range(3):
        e.step(4)
        pos = e.download()["pos"]
        assert e.pair_count() == brute_pairs(pos, box)
    e.close()
