"""The autotuner's host logic (no GPU): choice of the fastest (reach, skin),
then of the fastest force-pass shape (lanes, blocks) at it, then of the
density pass's lanes (with kept lists), skipping choices the box refuses,
and the JSON cache per signature."""
import json

import pytest

from implicit_dpd_gb300 import autotune as A


class FakeEngine:
    """Step times per (reach, skin), scaled per force-pass shape by
    shape_ms; skins above max_skin are refused like a box too small for
    them."""

    def __init__(self, ms, max_skin=1.0, shape_ms=None, dens_ms=None):
        self.ms, self.max_skin = ms, max_skin
        self.shape_ms = shape_ms or {}
        self.dens_ms = dens_ms or {}
        self.tuning, self.shape, self.dens, self.steps, self.last = None, None, None, 0, 0.0

    def set_tuning(self, reach, skin=0.0, lanes=16, blocks=1, dens_lanes=32):
        if skin > self.max_skin:
            raise ValueError("skin needs a larger box")
        self.tuning = (reach, skin)
        self.shape = (lanes, blocks)
        self.dens = dens_lanes

    def step(self, n):
        self.steps += n
        self.last = (self.ms[self.tuning] * self.shape_ms.get(self.shape, 1.0) *
                     self.dens_ms.get(self.dens, 1.0) * n)

    def last_step_ms(self):
        return self.last


def test_picks_the_fastest_and_applies_it():
    ms = {c: 5.0 for c in A.DEFAULT_CHOICES}
    ms[(1, 0.15)] = 3.2
    e = FakeEngine(ms)
    choice, times = A.tune(e)
    assert choice == {"reach": 1, "skin": 0.15, "lanes": 16, "blocks": 1, "dens_lanes": 32}
    assert e.tuning == (1, 0.15) and e.shape == (16, 1) and e.dens == 32
    assert times["reach1_skin0.15"] == pytest.approx(3.2)
    assert len(times) == len(A.DEFAULT_CHOICES) + len(A.SHAPES) + len(A.DENS_LANES)


def test_then_picks_the_fastest_force_shape_at_that_reach_and_skin():
    ms = {c: 5.0 for c in A.DEFAULT_CHOICES}
    ms[(2, 0.2)] = 3.0
    e = FakeEngine(ms, shape_ms={(8, 1): 0.9, (32, 1): 1.2})
    choice, times = A.tune(e)
    assert choice == {"reach": 2, "skin": 0.2, "lanes": 8, "blocks": 1, "dens_lanes": 32}
    assert e.tuning == (2, 0.2) and e.shape == (8, 1)
    assert times["lanes8_blocks1"] == pytest.approx(2.7)


def test_then_picks_the_density_lanes_with_kept_lists_only():
    ms = {c: 5.0 for c in A.DEFAULT_CHOICES}
    ms[(1, 0.2)] = 3.0
    e = FakeEngine(ms, dens_ms={8: 0.8, 16: 0.9})
    choice, times = A.tune(e)
    assert choice["dens_lanes"] == 8 and e.dens == 8
    assert times["dens_lanes8"] == pytest.approx(2.4)
    # at skin 0 the density pass sweeps the cells: its lanes are not timed
    ms = {c: 5.0 for c in A.DEFAULT_CHOICES}
    ms[(1, 0.0)] = 2.0
    choice, times = A.tune(FakeEngine(ms, dens_ms={8: 0.5}))
    assert choice["dens_lanes"] == 32 and "dens_lanes8" not in times


def test_skips_choices_the_box_refuses():
    ms = {c: 4.0 - c[1] for c in A.DEFAULT_CHOICES}  # larger skins faster
    e = FakeEngine(ms, max_skin=0.15)
    choice, times = A.tune(e)
    assert choice["skin"] == 0.15
    assert all(float(k.split("skin")[1]) <= 0.15 for k in times if k.startswith("reach"))
    with pytest.raises(ValueError):
        A.tune(FakeEngine(ms, max_skin=-1.0))


def test_cache_round_trip(tmp_path):
    path = str(tmp_path / "sub" / "tuning.json")
    key = A.signature("GB300", 984040, 64 * 64 * 48, 0)
    ms = {c: 5.0 for c in A.DEFAULT_CHOICES}
    ms[(2, 0.2)] = 2.0
    e = FakeEngine(ms)
    A.tune(e, key=key, cache_path=path)
    stored = json.load(open(path))
    assert stored[key]["reach"] == 2 and stored[key]["skin"] == 0.2
    e2 = FakeEngine(ms)
    choice, times = A.tune(e2, key=key, cache_path=path)
    assert choice == {"reach": 2, "skin": 0.2, "lanes": 16, "blocks": 1, "dens_lanes": 32}
    assert times == {} and e2.steps == 0 and e2.shape == (16, 1)
    ms[(1, 0.1)] = 1.0
    choice, times = A.tune(FakeEngine(ms, shape_ms={(16, 2): 0.5}), key=key, cache_path=path,
                           refresh=True)
    assert choice == {"reach": 1, "skin": 0.1, "lanes": 16, "blocks": 2, "dens_lanes": 32}
    assert json.load(open(path))[key]["skin"] == 0.1 and json.load(open(path))[key]["blocks"] == 2


def test_signature_groups_close_systems():
    a = A.signature("GB300", 1_000_000, 196_608, 0)
    b = A.signature("GB300", 1_020_000, 200_000, 0)
    c = A.signature("GB300", 2_000_000, 196_608, 0)
    assert a == b and a != c and a != A.signature("GB300", 1_000_000, 196_608, 2)
