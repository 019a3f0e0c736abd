"""idpd_step(h, K) sends the K steps to the device in one graph launch (the
step inside a conditional WHILE node) instead of one launch per step. The
kernels and their order are the same, so the state after K steps must be
the same bit for bit, with and without kept lists, across storage reorders
that fall inside the K steps, for batched replicas, and with the reaction
enabled (the loop ends on the device after the step whose event stopped the
run)."""
import numpy as np
import pytest

from helpers import mdpd_params, mixed_system
from implicit_dpd_gb300 import configs
from implicit_dpd_gb300.abi import CFG_PLAIN_GRAPHS, FORM_WARREN
from implicit_dpd_gb300.engine import Engine, EngineError, derive_params

pytestmark = pytest.mark.gpu


def _run(flags, skin, sort_period, chunks):
    box, st, n_amp = mixed_system(seed=31)
    e = Engine(flags=flags, sort_period=sort_period)
    e.set_params(mdpd_params(box, time=9))
    e.upload(st)
    e.build_topology(n_amp, [0, 3])
    e.set_tuning(1, skin)
    for k in chunks:
        e.step(k)
    out = e.download()
    rebuilds = e.list_rebuilds()
    t = e.get_params().time
    e.close()
    return out, rebuilds, t


@pytest.mark.parametrize("skin,sort_period", [(0.0, 100), (0.25, 7), (0.15, 3)])
def test_one_launch_for_k_steps_equals_one_launch_per_step(skin, sort_period):
    chunks = [1, 9, 4, 13]
    a, ra, ta = _run(0, skin, sort_period, chunks)
    b, rb, tb = _run(CFG_PLAIN_GRAPHS, skin, sort_period, chunks)
    for k in ("pos", "vel", "acc", "id", "prop"):
        assert np.array_equal(a[k], b[k]), k
    assert ra == rb and ta == tb == 9 + sum(chunks)


def test_batched_replicas_one_launch():
    reps = configs.mdpd_replicas(6, seed=4, n_min=800, n_max=3000)
    params = []
    for r in reps:
        q = derive_params(configs.run_param(r["box"], dt=0.005, cf_r=3.0))
        q.seed, q.time, q.form = r["seed"], 1, FORM_WARREN
        q.warren_a, q.warren_b, q.warren_rd = r["a"], 25.0, 0.75
        params.append(q)

    def run(flags):
        e = Engine(n_replicas=len(reps), flags=flags, sort_period=5)
        for k, (r, q) in enumerate(zip(reps, params)):
            e.set_params(q, k)
            e.upload(r["state"], k)
        e.set_tuning(1, 0.2)
        e.step(12)
        out = [e.download(replica=k) for k in range(len(reps))]
        e.close()
        return out

    a, b = run(0), run(CFG_PLAIN_GRAPHS)
    for x, y in zip(a, b):
        assert np.array_equal(x["pos"], y["pos"]) and np.array_equal(x["vel"], y["vel"])


def test_reaction_in_one_launch_stops_where_the_steps_do():
    # the reaction's event runs inside the loop; the loop ends after the step
    # whose event reached max_amp_num, as the one-launch-per-step form does
    from implicit_dpd_gb300.abi import IdpdChemParams
    import pyoracle as O

    box = np.array([10.0, 10.0, 10.0])
    n_amp = 600
    st = configs.flat_bilayers(box, n_amp, seed=5, jitter=0.05)
    core = [0, 1, 7]
    core_ptcl = [int(st["id"][(st["amp_id"] == a) & (st["unit"] == 0)][0]) for a in core]

    def run(flags):
        p = O.derive_params(configs.run_param(box, cf_b_rigid=20.0))
        p.seed, p.time = 1, 5
        cp = IdpdChemParams(p_thresld=0.3, eps=0.2, influ_rad=2.0, influ_hei=0.8, influ_dep=4.0,
                            influ_grd=-0.5, amp_num=n_amp, max_amp_num=640)
        e = Engine(flags=flags, sort_period=4)
        e.set_params(p)
        e.upload(st)
        e.build_topology(n_amp, core)
        e.set_chem(cp, 1234, core_ptcl, 200, beg_chem=6)
        stopped = False
        for k in (3, 8, 8, 8, 8):
            try:
                e.step(k)
            except EngineError:
                stopped = True
                break
        out = e.download()
        t = e.get_params().time
        e.close()
        return out, t, stopped

    (a, ta, sa), (b, tb, sb) = run(0), run(CFG_PLAIN_GRAPHS)
    assert sa == sb and ta == tb
    assert len(a["pos"]) == len(b["pos"]) > len(st["pos"])
    for k in ("pos", "vel", "acc", "id", "prop", "amp_id", "unit"):
        assert np.array_equal(a[k], b[k]), k


def test_observing_steps_between_loop_launches():
    # with observations every 4 steps, the steps between them go in loop
    # launches and each observing step in the observation graph: the records
    # and the state equal those of one launch per step
    def run(flags):
        box, st, n_amp = mixed_system(seed=41)
        e = Engine(flags=flags, sort_period=6)
        e.set_params(mdpd_params(box, time=2))
        e.upload(st)
        e.build_topology(n_amp, [0, 3])
        e.set_tuning(1, 0.2)
        e.set_observe(4)
        for k in (5, 11, 1, 9):
            e.step(k)
        obs = e.observations()
        out = e.download()
        e.close()
        return obs, out

    (oa, a), (ob, b) = run(0), run(CFG_PLAIN_GRAPHS)
    assert len(oa) == len(ob) > 0
    assert [o["time"] for o in oa] == [o["time"] for o in ob]
    for x, y in zip(oa, ob):
        for k in x:
            assert np.array_equal(np.asarray(x[k]), np.asarray(y[k])), k
    for k in ("pos", "vel", "acc"):
        assert np.array_equal(a[k], b[k]), k
