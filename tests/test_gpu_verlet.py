"""Kept neighbour lists (idpd_tuning.skin > 0): the engine rebuilds cells and
lists only when a particle has moved more than half the skin. Every step
must still see exactly the reference's pair set, so each step is compared
with one oracle step from the engine's own state (drift bit-exact, forces
within 1e-5), across rebuild and non-rebuild steps, storage reorders and
periodic wraps."""
import numpy as np
import pytest

import pyoracle as O
from helpers import FORCE_TOL, mdpd_params, mixed_system, rel_force_err
from implicit_dpd_gb300.engine import Engine, EngineError

pytestmark = pytest.mark.gpu


def _engine(p, st, n_amp, skin, sort_period=0, reach=1):
    e = Engine(sort_period=sort_period)
    e.set_params(p)
    e.upload(st)
    e.build_topology(n_amp, [0, 3])
    e.set_tuning(reach, skin)
    return e


def _oracle_step(p, s0, n_amp, time):
    ref = {k: s0[k].copy() for k in ("pos", "vel", "acc", "id", "prop")}
    ref["topol"], ref["cf_bend"] = O.build_topology(s0["amp_id"], s0["unit"], n_amp, [0, 3], p.cf_b,
                                                    p.cf_b_rigid)
    po = type(p).from_buffer_copy(p)
    po.time = time
    O.md_step(po, ref, nthreads=4)
    return ref


@pytest.mark.parametrize("skin,sort_period,reach", [(0.3, 0, 1), (0.3, 7, 1), (0.15, 5, 1),
                                                    (0.3, 0, 2), (0.2, 5, 2)])
def test_kept_lists_give_the_reference_step(skin, sort_period, reach):
    box, st, n_amp = mixed_system(seed=9)
    p = mdpd_params(box, time=60)
    e = _engine(p, st, n_amp, skin, sort_period, reach)
    assert abs(e.get_skin() - skin) < 1e-7
    done = 0
    for target in (0, 1, 12, 45):
        e.step(target - done)
        done = target
        s0 = e.download()
        t0 = e.get_params().time
        e.step(1)
        done += 1
        s1 = e.download()
        ref = _oracle_step(p, s0, n_amp, t0)
        assert np.array_equal(s1["pos"], ref["pos"]), target
        assert rel_force_err(s1["acc"], ref["acc"])[0] < FORCE_TOL, target
        f_rms = np.sqrt((ref["acc"] ** 2).sum(1).mean())
        assert np.abs(s1["vel"] - ref["vel"]).max() < 0.5 * p.dt * FORCE_TOL * f_rms + 1e-12


def test_kept_lists_follow_the_plain_trajectory():
    box, st, n_amp = mixed_system(seed=2)
    p = mdpd_params(box, time=5)
    out = []
    for skin, reach in ((0.0, 1), (0.3, 1), (0.3, 2)):
        e = _engine(p, st, n_amp, skin, reach=reach)
        e.step(40)
        out.append(e.download())
    for o in out[1:]:
        assert np.abs(out[0]["pos"] - o["pos"]).max() < 1e-6
        assert rel_force_err(o["acc"], out[0]["acc"])[1] < 1e-4
    # the reach changes neither the pair sets nor the fixed-point sums
    assert np.array_equal(out[1]["pos"], out[2]["pos"])
    assert np.array_equal(out[1]["acc"], out[2]["acc"])


def test_skin_needs_room_in_the_box():
    box, st, n_amp = mixed_system(box=(9.0, 10.0, 11.0))
    e = Engine()
    e.set_params(mdpd_params(box))
    with pytest.raises(EngineError, match="skin"):
        e.set_tuning(1, 2.5)


@pytest.mark.parametrize("skin", [0.0, 0.3])
def test_host_roundtrip_keeps_the_trajectory(skin):
    """Positions, velocities and accelerations read back and handed in again
    every step (the per-step host exchange) change nothing: the kept lists
    stay (the position change is zero) and the states agree bit for bit."""
    box, st, n_amp = mixed_system(seed=21)
    p = mdpd_params(box, time=40)
    a = _engine(p, st, n_amp, skin)
    a.step(12)
    b = _engine(p, st, n_amp, skin)
    n = len(st["pos"])
    pos, vel, acc = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
    for _ in range(12):
        b.download_dynamics(pos, vel, acc)
        b.set_dynamics(pos, vel, acc)
        b.step(1)
    sa, sb = a.download(), b.download()
    for k in ("pos", "vel", "acc"):
        assert np.array_equal(sa[k], sb[k]), k
    assert a.list_rebuilds() == b.list_rebuilds()


def test_host_move_past_half_the_skin_rebuilds():
    """A particle moved by the host by more than half the skin (across the
    periodic boundary) makes the next step rebuild, and that step matches the
    oracle step from the state handed in."""
    box, st, n_amp = mixed_system(seed=22)
    p = mdpd_params(box, time=70)
    e = _engine(p, st, n_amp, 0.2)
    e.step(5)
    s = e.download()
    k = int(np.argmin(s["pos"][:, 0]))
    pos = s["pos"].copy()
    pos[k, 0] = np.mod(pos[k, 0] - 0.35, box[0])  # wraps to the far side
    e.set_dynamics(pos, s["vel"], s["acc"])
    r0 = e.list_rebuilds()
    s0 = e.download()
    assert np.array_equal(s0["pos"], pos)
    t0 = e.get_params().time
    e.step(1)
    assert e.list_rebuilds() == r0 + 1
    s1 = e.download()
    ref = _oracle_step(p, s0, n_amp, t0)
    assert np.array_equal(s1["pos"], ref["pos"])
    assert rel_force_err(s1["acc"], ref["acc"])[0] < FORCE_TOL


def test_exchange_through_pinned_and_device_buffers():
    """Page-locked host buffers go through the copy engines like pageable
    ones; device buffers are read and written by the kernels where they lie.
    All three give the same states bit for bit."""
    torch = pytest.importorskip("torch")
    box, st, n_amp = mixed_system(seed=23)
    p = mdpd_params(box, time=50)
    runs = []
    for kind in ("numpy", "pinned", "device"):
        e = _engine(p, st, n_amp, 0.3)
        e.step(4)
        n = len(st["pos"])
        if kind == "numpy":
            bufs = [np.zeros((n, 3)) for _ in range(3)]
        elif kind == "pinned":
            bufs = [torch.zeros((n, 3), dtype=torch.float64, pin_memory=True) for _ in range(3)]
        else:
            bufs = [torch.zeros((n, 3), dtype=torch.float64, device="cuda") for _ in range(3)]
        for _ in range(3):
            e.download_dynamics(*bufs)
            if kind == "device":
                torch.cuda.synchronize()
            e.set_dynamics(*bufs)
            e.step(1)
        e.download_dynamics(*bufs)
        torch.cuda.synchronize()
        out = [b.cpu().numpy() if hasattr(b, "cpu") else b for b in bufs]
        assert np.array_equal(out[0], e.download()["pos"]), kind
        runs.append(out)
    for k in range(3):
        assert np.array_equal(runs[0][k], runs[1][k])
        assert np.array_equal(runs[0][k], runs[2][k])
