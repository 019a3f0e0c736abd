"""Edge cases of the step: an empty replica among others, a lone particle,
particles on the box faces (x = 0 and x = L, both accepted by the upload and
wrapped by the reference's floor expression), nearly coincident and
near-cutoff pairs, and a box of three cells per side."""
import numpy as np
import pytest

import pyoracle as O
from helpers import FORCE_TOL, mdpd_params, mixed_system, rel_force_err
from implicit_dpd_gb300 import configs
from implicit_dpd_gb300.abi import SOLVENT
from implicit_dpd_gb300.engine import Engine

pytestmark = pytest.mark.gpu


def engine_for(p, st, n_amp=0, core=()):
    e = Engine()
    e.set_params(p)
    e.upload(st)
    if n_amp:
        e.build_topology(n_amp, core)
    return e


def _oracle_step(p, s0, t0):
    po = type(p).from_buffer_copy(p)
    po.time = t0
    ref = {k: s0[k].copy() for k in ("pos", "vel", "acc", "id", "prop")}
    O.md_step(po, ref, nthreads=4)
    return ref


def _single(pos, box, vel=None):
    n = len(pos)
    none = np.full(n, 0xFFFFFFFF, np.uint32)
    return {"pos": np.asarray(pos, np.float64), "vel": np.zeros((n, 3)) if vel is None else vel,
            "acc": np.zeros((n, 3)), "id": np.arange(n, dtype=np.uint32),
            "prop": np.full(n, SOLVENT, np.uint32), "amp_id": none, "unit": none.copy()}


def _step_vs_oracle(p, st, steps=1):
    e = engine_for(p, st)
    for _ in range(steps):
        s0 = e.download()
        t0 = e.get_params().time
        e.step(1)
        s1 = e.download()
        ref = _oracle_step(p, s0, t0)
        assert np.array_equal(s1["pos"], ref["pos"])
        if np.any(ref["acc"] != 0.0):
            assert rel_force_err(s1["acc"], ref["acc"])[0] < FORCE_TOL
        else:
            assert np.array_equal(s1["acc"], ref["acc"])
        assert np.array_equal(s1["vel"], ref["vel"]) or np.any(ref["acc"] != 0.0)
    return e


def test_empty_replica_among_others():
    box, st, n_amp = mixed_system(seed=41, box=(8.0, 8.0, 8.0), n_amp=200)
    empty = _single(np.zeros((0, 3)), box)
    p = mdpd_params(box, seed=3, time=9)
    e = Engine(n_replicas=3)
    for k, s in enumerate([st, empty, st]):
        e.set_params(p, k)
        e.upload(s, k)
        if len(s["pos"]):
            e.build_topology(n_amp, [0], k)
    e.step(3)
    assert e.num_particles(1) == 0
    single = engine_for(p, st, n_amp, [0])
    single.step(3)
    want = single.download()
    for k in (0, 2):
        got = e.download(k)
        for key in ("pos", "vel", "acc"):
            assert np.array_equal(got[key], want[key]), (k, key)


def test_lone_particle_drifts_without_force():
    box = np.array([5.0, 5.0, 5.0])
    st = _single([[2.5, 2.5, 2.5]], box, vel=np.array([[0.3, -0.2, 0.1]]))
    p = mdpd_params(box, time=2)
    e = _step_vs_oracle(p, st, steps=3)
    assert np.all(e.download()["acc"] == 0.0)


def test_particles_on_the_box_faces_and_coincident_pairs():
    box = np.array([6.0, 7.0, 8.0])
    rng = np.random.default_rng(3)
    pos = rng.random((600, 3)) * box
    pos[:20, 0] = 0.0          # on the lower face
    pos[20:40, 1] = box[1]     # on the upper face: the drift's floor wraps it
    pos[40:45] = pos[45:50]    # coincident pairs of distinct particles
    pos[50, :] = pos[51, :] + np.array([1.0 - 1e-12, 0.0, 0.0])  # a pair a hair inside the cutoff
    pos[52, :] = pos[53, :] + np.array([0.0, 1.0, 0.0])          # exactly at the cutoff
    pos = np.mod(pos, box)
    pos[20:40, 1] = box[1]
    st = _single(pos, box, vel=rng.normal(size=(600, 3)))
    p = mdpd_params(box, time=17)
    # coincident particles have no pair direction: the reference divides by zero
    st["pos"][40:45] += 1e-7
    _step_vs_oracle(p, st, steps=2)


def test_smallest_box_three_cells_per_side():
    box = np.array([3.61, 3.7, 3.95])  # three cells per side for the engine and the oracle
    st = configs.liquid(box, 4.0, seed=8)
    p = mdpd_params(box, time=4)
    _step_vs_oracle(p, st, steps=3)
