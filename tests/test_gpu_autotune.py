"""The package's tuner on a real handle: every (reach, skin) the box allows is
timed and the rest skipped, the fastest choice is applied and cached, a
cached choice is applied without timing, and a step of the tuned handle
matches the oracle's step."""
import json

import numpy as np
import pytest

import pyoracle as O
from helpers import FORCE_TOL, mdpd_params, rel_force_err
from implicit_dpd_gb300 import autotune as A
from implicit_dpd_gb300 import configs
from implicit_dpd_gb300.engine import Engine

pytestmark = pytest.mark.gpu


def _liquid(box):
    st = configs.liquid(box, 4.0, seed=9)
    st["id"] = np.arange(len(st["pos"]), dtype=np.uint32)
    return st


def test_tune_applies_caches_and_keeps_the_forces(tmp_path):
    # box side 4: skins above 1/3 leave fewer than three cells of 1 + skin
    box = np.array([4.0, 4.0, 4.0])
    st = _liquid(box)
    p = mdpd_params(box, time=3)
    e = Engine()
    e.set_params(p)
    e.upload(st)
    e.step(2)
    path = str(tmp_path / "tuning.json")
    key = A.signature("test", len(st["pos"]), float(np.prod(box)), int(p.form))
    choice, times = A.tune(e, steps=4, key=key, cache_path=path, rounds=1)
    allowed = [c for c in A.DEFAULT_CHOICES if 3.0 * (1.0 + c[1]) <= 4.0]
    refused = [c for c in A.DEFAULT_CHOICES if c not in allowed]
    assert refused and all(f"reach{r}_skin{s:g}" not in times for r, s in refused)
    assert all(f"reach{r}_skin{s:g}" in times for r, s in allowed)
    assert all(f"lanes{l}_blocks{b}" in times for l, b in A.SHAPES)
    assert e.tuning() == {"reach": choice["reach"], "skin": round(choice["skin"], 6),
                          "lanes": choice["lanes"], "blocks": choice["blocks"],
                          "dens_lanes": choice["dens_lanes"]}
    cached = json.load(open(path))[key]
    assert {k: cached[k] for k in choice} == choice
    # a second handle of the same workload takes the cached choice untimed
    f = Engine()
    f.set_params(p)
    f.upload(st)
    choice2, times2 = A.tune(f, key=key, cache_path=path)
    assert choice2 == choice and times2 == {}
    assert f.tuning() == e.tuning()
    # a step of the tuned handle against the oracle's step from the same state
    s0 = f.download()
    q = type(p).from_buffer_copy(p)
    q.time = f.get_params().time
    f.step(1)
    s1 = f.download()
    ref = {k: s0[k].copy() for k in ("pos", "vel", "acc", "id", "prop")}
    O.md_step(q, ref, nthreads=4)
    assert np.array_equal(s1["pos"], ref["pos"])
    assert rel_force_err(s1["acc"], ref["acc"])[0] < FORCE_TOL
    e.close()
    f.close()
