"""Launch shapes of the force pass (idpd_tuning.pair_lanes, pair_blocks):
lanes per particle 4, 8, 16 or 32 and 1, 2 or 4 row blocks per CTA, and the
density pass's lanes per particle over kept lists (density_lanes). Every
shape evaluates the same pairs into the same fixed-point sums, so forces and
trajectories must be equal bit for bit; a CTA whose row blocks belong to
different replicas (and pair forms) must keep each block's tables."""
import numpy as np
import pytest

from helpers import FORCE_TOL, mdpd_params, mixed_system, oracle_forces, rel_force_err, warren_params
from implicit_dpd_gb300 import configs
from implicit_dpd_gb300.engine import Engine, EngineError

pytestmark = pytest.mark.gpu
SHAPES = [(16, 1), (8, 1), (32, 1), (16, 2), (16, 4), (8, 4), (32, 2), (4, 1), (4, 2)]


def test_density_lanes_give_the_same_trajectory():
    # the density pass over kept lists with 32, 16 or 8 lanes per particle:
    # the same densities, pass-2 lists and hence trajectories bit for bit
    box, st, n_amp = mixed_system(seed=23)
    p = mdpd_params(box, time=13)
    out = []
    for dl in (32, 16, 8, 4):
        e = Engine(sort_period=9)
        e.set_params(p)
        e.upload(st)
        e.build_topology(n_amp)
        e.set_tuning(1, 0.2, dens_lanes=dl)
        assert e.tuning()["dens_lanes"] == dl
        e.step(30)
        out.append((e.download(), e.list_rebuilds(), e.pair_count()))
        e.close()
    for (s, rb, pc), dl in zip(out[1:], (16, 8, 4)):
        for k in ("pos", "vel", "acc"):
            assert np.array_equal(s[k], out[0][0][k]), (dl, k)
        assert rb == out[0][1] and pc == out[0][2], dl
    # Warren liquids in a batched handle
    reps = [configs.liquid(np.array([7.0, 7.5, 8.0]), 5.0, seed=s) for s in (1, 2)]
    res = []
    for dl in (32, 4):
        e = Engine(n_replicas=2)
        for r, rs in enumerate(reps):
            e.set_params(warren_params(np.array([7.0, 7.5, 8.0]), seed=5 + r), replica=r)
            e.upload(rs, replica=r)
        e.set_tuning(1, 0.25, dens_lanes=dl)
        e.step(20)
        res.append([e.download(replica=r)["pos"] for r in range(2)])
        e.close()
    assert all(np.array_equal(a, b) for a, b in zip(res[0], res[1]))


def test_every_shape_gives_the_same_forces_and_trajectory():
    box, st, n_amp = mixed_system(seed=21)
    p = mdpd_params(box, time=11)
    _, _, _, acc, _ = oracle_forces(p, st)
    out = []
    for lanes, blocks in SHAPES:
        e = Engine()
        e.set_params(p)
        e.upload(st)
        e.build_topology(n_amp)
        e.set_tuning(1, 0.0, lanes=lanes, blocks=blocks)
        assert e.tuning()["lanes"] == lanes and e.tuning()["blocks"] == blocks
        e.density()
        e.force()
        f = e.download()["acc"]
        assert rel_force_err(f, acc)[0] < FORCE_TOL, (lanes, blocks)
        e.set_tuning(1, 0.2)
        e.step(25)
        out.append((f, e.download()))
        e.close()
    for (f, s), shape in zip(out[1:], SHAPES[1:]):
        assert np.array_equal(f, out[0][0]), shape
        assert np.array_equal(s["pos"], out[0][1]["pos"]), shape
        assert np.array_equal(s["acc"], out[0][1]["acc"]), shape


def test_mixed_replicas_in_one_cta():
    """Three small replicas (MDPD, Warren, MDPD) whose row blocks share CTAs
    at 4 blocks per CTA: the batch equals each replica run alone."""
    systems = []
    for k in range(3):
        box = np.array([6.0 + k, 6.5, 7.0])
        st = configs.liquid(box, 5.0 + k, seed=30 + k)
        p = warren_params(box, seed=7 + k) if k == 1 else mdpd_params(box, seed=7 + k)
        systems.append((box, st, p))
    alone = []
    for box, st, p in systems:
        e = Engine()
        e.set_params(p)
        e.upload(st)
        e.step(5)
        alone.append(e.download()["acc"])
        e.close()
    for lanes, blocks in ((16, 4), (8, 2), (32, 4)):
        e = Engine(n_replicas=3)
        for k, (box, st, p) in enumerate(systems):
            e.set_params(p, k)
            e.upload(st, k)
        e.set_tuning(1, 0.0, lanes=lanes, blocks=blocks)
        e.step(5)
        for k in range(3):
            assert np.array_equal(e.download(k)["acc"], alone[k]), (lanes, blocks, k)
        e.close()


def test_shape_arguments_are_checked():
    box, st, _ = mixed_system()
    e = Engine()
    e.set_params(mdpd_params(box))
    with pytest.raises(EngineError, match="pair_lanes"):
        e.set_tuning(1, 0.0, lanes=12)
    with pytest.raises(EngineError, match="pair_blocks"):
        e.set_tuning(1, 0.0, blocks=3)
    e.close()
