"""The precursor conversion of the membrane-with-precursor workload: a
precursor bead (here the solvent beads) with a tail bead within the cutoff
converts to a head when its Saru(id, time, seed) draw is below the
threshold. Each engine step is compared with the oracle's decisions taken
from the engine's own state, bit for bit, through the cell sweep (no kept
lists), the kept lists, the FP64 arm (cell sweep) and a cluster whose pair
lists overflow; a replica without the conversion is left alone."""
import numpy as np
import pytest

import pyoracle as O
from helpers import mdpd_params, mixed_system
from implicit_dpd_gb300.abi import (CFG_FP64_PAIRS, HYPHIL, HYPHOB, SOLVENT,
                                    precursor_threshold)
from implicit_dpd_gb300.engine import Engine

pytestmark = pytest.mark.gpu
SEED = 4242


def _engine(p, st, n_amp, flags=0, skin=0.0, dens_lanes=32):
    e = Engine(flags=flags)
    e.set_params(p)
    e.upload(st)
    e.build_topology(n_amp, [0, 3])
    if skin:
        e.set_tuning(1, skin, dens_lanes=dens_lanes)
    return e


def _check_steps(e, p, steps, thr):
    total = 0
    for _ in range(steps):
        s0 = e.download()
        t0 = e.get_params().time
        e.step(1)
        s1 = e.download()
        # the step decides on its drifted positions (the kick moves none) and
        # on the properties it started with
        want, cnt = O.precursor(p, s1["pos"], s1["id"], s0["prop"], t0, SOLVENT, HYPHOB, HYPHIL,
                                thr, SEED, nthreads=4)
        assert np.array_equal(s1["prop"], want), t0
        total += cnt
    assert e.precursor_count() == total
    return total


@pytest.mark.parametrize("flags,skin,dens_lanes", [(0, 0.0, 32), (0, 0.2, 32), (0, 0.2, 16),
                                                   (0, 0.2, 8), (0, 0.2, 4),
                                                   (CFG_FP64_PAIRS, 0.0, 32)])
def test_precursor_decisions_match_oracle(flags, skin, dens_lanes):
    box, st, n_amp = mixed_system(seed=12)
    p = mdpd_params(box, time=300)
    thr = precursor_threshold(0.05)
    e = _engine(p, st, n_amp, flags, skin, dens_lanes)
    e.set_precursor(SOLVENT, HYPHOB, HYPHIL, thr, SEED)
    total = _check_steps(e, p, 6, thr)
    assert total > 20


def test_precursor_through_an_overflowed_list():
    """700 precursors packed within 0.8 of a tail bead: the tail bead and most
    of the precursors have more than 512 pairs within the cutoff, so pass 1
    keeps no list for them and pass 2 walks their cells."""
    box, st, n_amp = mixed_system(seed=13)
    NB = 700
    rng = np.random.default_rng(5)
    tail = int(np.flatnonzero(st["prop"] == HYPHOB)[0])
    v = rng.normal(size=(NB, 3))
    v *= (0.8 * rng.random(NB) ** (1 / 3) / np.linalg.norm(v, axis=1))[:, None]
    blob = np.mod(st["pos"][tail] + v, box)
    n0 = len(st["pos"])
    st = dict(st)
    st["pos"] = np.concatenate([st["pos"], blob])
    st["vel"] = np.concatenate([st["vel"], np.zeros((NB, 3))])
    st["acc"] = np.concatenate([st["acc"], np.zeros((NB, 3))])
    st["prop"] = np.concatenate([st["prop"], np.full(NB, SOLVENT, np.uint32)])
    for k in ("amp_id", "unit"):
        st[k] = np.concatenate([st[k], np.full(NB, 0xFFFFFFFF, np.uint32)])
    st["id"] = np.arange(n0 + NB, dtype=np.uint32)
    p = mdpd_params(box, time=31)
    thr = precursor_threshold(0.5)
    e = _engine(p, st, n_amp)
    e.set_precursor(SOLVENT, HYPHOB, HYPHIL, thr, SEED)
    assert _check_steps(e, p, 1, thr) > 50


def test_precursor_off_and_per_replica():
    box, st, n_amp = mixed_system(seed=14)
    p = mdpd_params(box, time=5)
    e = Engine(n_replicas=2)
    for r in range(2):
        e.set_params(p, r)
        e.upload(st, r)
        e.build_topology(n_amp, [0], r)
    e.set_precursor(SOLVENT, HYPHOB, HYPHIL, 0xFFFFFFFF, SEED, replica=1)
    e.step(2)
    assert np.array_equal(e.download(0)["prop"], st["prop"])
    assert e.precursor_count(0) == 0
    assert e.precursor_count(1) > 0
    changed = e.download(1)["prop"] != st["prop"]
    assert np.all(st["prop"][changed] == SOLVENT)
    e.set_precursor(SOLVENT, HYPHOB, HYPHIL, 0xFFFFFFFF, SEED, replica=1, enabled=False)
    before = e.download(1)["prop"]
    e.step(2)
    assert np.array_equal(e.download(1)["prop"], before)
