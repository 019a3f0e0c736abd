"""idpd_step_host: one step on host arrays in one call (the rows in, one step,
the rows out, with the positions copied back while the pair passes run)
must leave exactly the state of idpd_set_dynamics + idpd_step(1) +
idpd_download_state, step after step: with and without kept lists, across
list rebuilds and storage reorders, and on a batched handle."""
import numpy as np
import pytest

import pyoracle as O
from helpers import mdpd_params, mixed_system
from implicit_dpd_gb300 import configs
from implicit_dpd_gb300.abi import IdpdChemParams
from implicit_dpd_gb300.engine import Engine, EngineError

pytestmark = pytest.mark.gpu


def _engine(p, st, n_amp, skin, sort_period):
    e = Engine(sort_period=sort_period)
    e.set_params(p)
    e.upload(st)
    e.build_topology(n_amp, [0, 3])
    e.set_tuning(1, skin)
    return e


@pytest.mark.parametrize("skin,sort_period", [(0.0, 100), (0.3, 3), (0.15, 2)])
def test_step_host_equals_the_three_calls(skin, sort_period):
    box, st, n_amp = mixed_system(seed=21)
    p = mdpd_params(box, time=5)
    a = _engine(p, st, n_amp, skin, sort_period)
    b = _engine(p, st, n_amp, skin, sort_period)
    n = len(st["pos"])
    pa, va, aa = (np.ascontiguousarray(st[k], np.float64).copy() for k in ("pos", "vel", "acc"))
    pb, vb, ab = pa.copy(), va.copy(), aa.copy()
    for step in range(12):
        a.set_dynamics(pa, va, aa)
        a.step(1)
        a.download_dynamics(pa, va, aa)
        b.step_host(pb, vb, ab)
        for x, y, name in ((pa, pb, "pos"), (va, vb, "vel"), (aa, ab, "acc")):
            assert np.array_equal(x, y), f"{name} differs at step {step}"
    # the host copy is the device state
    out = b.download()
    assert np.array_equal(out["pos"], pb) and np.array_equal(out["acc"], ab)
    assert out["pos"].shape == (n, 3)
    if skin > 0:
        assert b.list_rebuilds() == a.list_rebuilds() and b.list_rebuilds() > 1
    a.close()
    b.close()


def test_step_host_with_observations():
    # observing steps go through the observation kernels in both forms; the
    # states and the drained records are the same bit for bit
    box, st, n_amp = mixed_system(seed=24)
    p = mdpd_params(box, time=4)
    a = _engine(p, st, n_amp, 0.2, 3)
    b = _engine(p, st, n_amp, 0.2, 3)
    for e in (a, b):
        e.set_observe(2)
    pa, va, aa = (np.ascontiguousarray(st[k], np.float64).copy() for k in ("pos", "vel", "acc"))
    pb, vb, ab = pa.copy(), va.copy(), aa.copy()
    for step in range(7):
        a.set_dynamics(pa, va, aa)
        a.step(1)
        a.download_dynamics(pa, va, aa)
        b.step_host(pb, vb, ab)
        for x, y, name in ((pa, pb, "pos"), (va, vb, "vel"), (aa, ab, "acc")):
            assert np.array_equal(x, y), f"{name} differs at step {step}"
    oa, ob = a.observations(), b.observations()
    assert len(oa) == len(ob) >= 3
    for x, y in zip(oa, ob):
        assert x["time"] == y["time"] and x["time"] % 2 == 0
        for k in ("kin_temp", "pressure", "diffusion"):
            assert np.array_equal(x[k], y[k]), k
    a.close()
    b.close()


def test_step_host_with_the_precursor_conversion():
    # the conversion changes properties on the device during the step; the
    # host exchange carries pos/vel/acc only, and both forms convert the same
    # particles
    from implicit_dpd_gb300.abi import HYPHIL, HYPHOB, SOLVENT, precursor_threshold
    box, st, n_amp = mixed_system(seed=12)
    p = mdpd_params(box, time=300)
    thr = precursor_threshold(0.05)
    a = _engine(p, st, n_amp, 0.2, 4)
    b = _engine(p, st, n_amp, 0.2, 4)
    for e in (a, b):
        e.set_precursor(SOLVENT, HYPHOB, HYPHIL, thr, 4242)
    pa, va, aa = (np.ascontiguousarray(st[k], np.float64).copy() for k in ("pos", "vel", "acc"))
    pb, vb, ab = pa.copy(), va.copy(), aa.copy()
    for step in range(6):
        a.set_dynamics(pa, va, aa)
        a.step(1)
        a.download_dynamics(pa, va, aa)
        b.step_host(pb, vb, ab)
        for x, y, name in ((pa, pb, "pos"), (va, vb, "vel"), (aa, ab, "acc")):
            assert np.array_equal(x, y), f"{name} differs at step {step}"
    assert a.precursor_count() == b.precursor_count() > 20
    assert np.array_equal(a.download()["prop"], b.download()["prop"])
    a.close()
    b.close()


def test_step_host_with_device_buffers():
    # device buffers are read and written by the kernels where they lie; the
    # result equals that of page-locked or pageable host arrays bit for bit
    torch = pytest.importorskip("torch")
    box, st, n_amp = mixed_system(seed=22)
    p = mdpd_params(box, time=9)
    a = _engine(p, st, n_amp, 0.2, 5)
    b = _engine(p, st, n_amp, 0.2, 5)
    host = [np.ascontiguousarray(st[k], np.float64).copy() for k in ("pos", "vel", "acc")]
    dev = [torch.from_numpy(x.copy()).to("cuda") for x in host]
    # before the first pass the rows are staged on the host: device buffers
    # go through copies there, in and out
    c = _engine(p, st, n_amp, 0.2, 5)
    out = [torch.zeros_like(x) for x in dev]
    c.download_dynamics(*out)
    c.set_dynamics(*dev)
    torch.cuda.synchronize()
    for x, y in zip(host, out):
        assert np.array_equal(x, y.cpu().numpy())
    c.close()
    for step in range(8):
        a.step_host(*host)
        b.step_host(*dev)
        torch.cuda.synchronize()
        for x, y in zip(host, dev):
            assert np.array_equal(x, y.cpu().numpy()), step
    a.close()
    b.close()


def _liquid_engine(st, box, skin):
    e = Engine(sort_period=4)
    e.set_params(mdpd_params(box, seed=17, time=2))
    e.upload(st)
    e.set_tuning(1, skin)
    return e


def test_step_host_with_host_moves():
    # 233k particles with kept lists and storage reorders every 4 steps; the
    # host moves particles between steps (small moves kept by the lists, one
    # large move that forces a rebuild)
    box = np.array([36.0, 36.0, 36.0])
    st = configs.liquid(box, 5.0, seed=31)
    st["id"] = np.arange(len(st["pos"]), dtype=np.uint32)
    a, b = _liquid_engine(st, box, 0.2), _liquid_engine(st, box, 0.2)
    pa, va, aa = (np.ascontiguousarray(st[k], np.float64).copy() for k in ("pos", "vel", "acc"))
    pb, vb, ab = pa.copy(), va.copy(), aa.copy()
    rng = np.random.default_rng(5)
    for step in range(10):
        if step in (4, 7):
            idx = rng.choice(len(pa), 1000, replace=False)
            shift = rng.uniform(-0.02, 0.02, size=(1000, 3))
            if step == 7:
                shift[0] = (0.3, 0.0, 0.0)  # beyond half the skin
            for p_ in (pa, pb):
                p_[idx] = np.mod(p_[idx] + shift, box)
        a.set_dynamics(pa, va, aa)
        a.step(1)
        a.download_dynamics(pa, va, aa)
        b.step_host(pb, vb, ab)
        for x, y, name in ((pa, pb, "pos"), (va, vb, "vel"), (aa, ab, "acc")):
            assert np.array_equal(x, y), f"{name} differs at step {step}"
        assert a.list_rebuilds() == b.list_rebuilds(), step
    assert b.list_rebuilds() >= 3
    a.close()
    b.close()


def test_step_host_on_a_batched_handle():
    # replica 1 is exchanged; both replicas step
    box = np.array([8.0, 8.0, 8.0])
    reps = [configs.liquid(box, 3.0, seed=s) for s in (3, 4)]
    for st in reps:
        st["id"] = np.arange(len(st["pos"]), dtype=np.uint32)

    def make():
        e = Engine(n_replicas=2)
        for r, st in enumerate(reps):
            e.set_params(mdpd_params(box, seed=11 + r, time=3), replica=r)
            e.upload(st, replica=r)
        e.set_tuning(1, 0.2)
        return e

    a, b = make(), make()
    st = reps[1]
    pa, va, aa = (np.ascontiguousarray(st[k], np.float64).copy() for k in ("pos", "vel", "acc"))
    pb, vb, ab = pa.copy(), va.copy(), aa.copy()
    for _ in range(6):
        a.set_dynamics(pa, va, aa, replica=1)
        a.step(1)
        a.download_dynamics(pa, va, aa, replica=1)
        b.step_host(pb, vb, ab, replica=1)
        assert np.array_equal(pa, pb) and np.array_equal(va, vb) and np.array_equal(aa, ab)
    assert np.array_equal(a.download(replica=0)["pos"], b.download(replica=0)["pos"])
    a.close()
    b.close()


def test_step_host_refuses_the_reaction():
    box = np.array([10.0, 10.0, 10.0])
    n_amp = 600
    st = configs.flat_bilayers(box, n_amp, seed=5, jitter=0.05)
    p = O.derive_params(configs.run_param(box))
    p.seed, p.time = 1, 5
    core = [int(st["id"][(st["amp_id"] == 0) & (st["unit"] == 0)][0])]
    cp = IdpdChemParams(p_thresld=0.3, eps=0.2, influ_rad=2.0, influ_hei=0.8, influ_dep=4.0,
                        influ_grd=-0.5, amp_num=n_amp, max_amp_num=700)
    e = Engine()
    e.set_params(p)
    e.upload(st)
    e.build_topology(n_amp, [0])
    e.set_chem(cp, 1234, core, 64)
    e.step(1)
    pos, vel, acc = (np.ascontiguousarray(st[k], np.float64).copy() for k in ("pos", "vel", "acc"))
    with pytest.raises(EngineError, match="reaction"):
        e.step_host(pos, vel, acc)
    e.close()
