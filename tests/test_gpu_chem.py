"""The reaction event (ChemManager::RandomChemEvent, LOCAL_CHEM_EVENT form) on
the GPU against the oracle's restatement (tests/test_oracle_golden.py pins
that restatement bit for bit to the reference's own chemmanager.hpp).

The event depends on the core geometry (GetCorePos: the core particle's
position and its neighbour centres of mass), which the engine sums in its own
order; the oracle is handed the engine's core geometry, and the geometry
itself is checked against the oracle's density pass to 1e-12. Given that,
the decisions (which molecules react, in which order) and the MT19937 stream
are bit-exact; new positions and velocities agree to 1e-12 (the device's
cos/sin/log differ from the host libm in the last bits).
"""
import numpy as np
import pytest

import pyoracle as O
from implicit_dpd_gb300 import configs
from implicit_dpd_gb300.abi import IdpdChemParams
from implicit_dpd_gb300.engine import Engine, EngineError

pytestmark = pytest.mark.gpu

BOX = np.array([10.0, 10.0, 10.0])
N_AMP = 600
CORE = [0, 1, 7]
RESERVE = 200
MT_SEED = 1234
FP_TOL = 1e-12


def _setup(p_thresld=0.3, max_amp_num=700, time=5, beg_chem=100000):
    st = configs.flat_bilayers(BOX, N_AMP, seed=5, jitter=0.05)
    p = O.derive_params(configs.run_param(BOX, cf_b_rigid=20.0))
    p.seed, p.time = 1, time
    core_ptcl = [int(st["id"][(st["amp_id"] == a) & (st["unit"] == 0)][0]) for a in CORE]
    cp = IdpdChemParams(p_thresld=p_thresld, eps=0.2, influ_rad=2.0, influ_hei=0.8, influ_dep=4.0,
                        influ_grd=-0.5, amp_num=N_AMP, max_amp_num=max_amp_num)
    e = Engine(sort_period=1000)
    e.set_params(p)
    e.upload(st)
    e.build_topology(N_AMP, CORE)
    e.set_chem(cp, MT_SEED, core_ptcl, RESERVE, beg_chem=beg_chem)
    return e, st, p, cp, core_ptcl


def _nei_cm_from_engine(st, info, core_ptcl):
    """nei_cm rows the oracle reads (GetCorePos): the engine's values at the
    core particles; checks the core position is the particle's own."""
    nei = np.zeros((len(st["pos"]), 6))
    for k, pid in enumerate(core_ptcl):
        row = int(np.nonzero(st["id"] == pid)[0][0])
        raw = info["core_raw"][k]
        assert np.array_equal(raw[:3], st["pos"][row])
        nei[row, :3] = raw[6:9]   # hydrophilic (nei_cm_pos[Hyphil])
        nei[row, 3:] = raw[3:6]   # hydrophobic (nei_cm_pos[Hyphob])
    return nei


def _compare_event(out, ref, n0, info, targets, amp):
    assert info["amp_num"] == amp
    assert np.array_equal(info["targets"], targets.astype(np.uint32))
    assert len(out["pos"]) == len(ref["pos"])
    for k in ("id", "prop", "amp_id", "unit"):
        assert np.array_equal(out[k], ref[k]), k
    assert np.abs(out["pos"][n0:] - ref["pos"][n0:]).max() < FP_TOL
    assert np.abs(out["vel"][n0:] - ref["vel"][n0:]).max() < FP_TOL


def test_core_geometry_matches_oracle_density():
    e, st, p, cp, core_ptcl = _setup(p_thresld=0.0)
    e.chem_event()
    info = e.chem_info()
    _, cm, _ = O.density(p, st["pos"], st["prop"], nthreads=4)
    for k, pid in enumerate(core_ptcl):
        row = int(np.nonzero(st["id"] == pid)[0][0])
        assert np.abs(info["core_raw"][k][6:9] - cm[row, :3]).max() < FP_TOL
        assert np.abs(info["core_raw"][k][3:6] - cm[row, 3:]).max() < FP_TOL
    assert info["n_targets"] == 0 and info["events"] == 1
    # h2t_vecs() / core_poss_h(): the unit head-to-tail vector and the
    # projected core position of DetermineTargetIdWithCorePos
    # (chemmanager.hpp:123-135) from the same core geometry
    box = np.asarray(BOX, np.float64)
    assert len(info["h2t"]) == len(core_ptcl) == len(info["core_h"])
    for k in range(len(core_ptcl)):
        raw = info["core_raw"][k]
        h2t = raw[3:6] - raw[:3]
        h2t -= box * np.round(h2t / box)
        h2t /= np.sqrt((h2t * h2t).sum())
        c2cm = raw[6:9] - raw[:3]
        c2cm -= box * np.round(c2cm / box)
        core_h = raw[:3] + (c2cm @ h2t) * h2t
        core_h -= np.floor(core_h / box) * box
        assert np.abs(info["h2t"][k] - h2t).max() < 1e-12
        assert np.abs(info["core_h"][k] - core_h).max() < 1e-12


def test_chem_event_decisions_bit_exact_two_events():
    """Two events in a row: the second continues the MT19937 stream and sees
    the molecules the first one added. Each oracle event starts from the
    engine's state before it (rows added by the engine differ from the
    oracle's in the last bits of cos/sin/log)."""
    e, st, p, cp, core_ptcl = _setup()
    mt = O.new_mt(MT_SEED)
    before = {k: st[k].copy() for k in ("pos", "vel", "acc", "id", "prop", "amp_id", "unit")}
    amp_num = N_AMP
    for event in range(2):
        cont = e.chem_event()
        info = e.chem_info()
        out = e.download()
        n0 = len(before["pos"])
        for k in before:  # existing rows untouched
            assert np.array_equal(out[k][:n0], before[k]), (event, k)
        nei = _nei_cm_from_engine(before, info, core_ptcl)
        topol, _ = O.build_topology(before["amp_id"], before["unit"], amp_num, CORE, p.cf_b,
                                    p.cf_b_rigid)
        cpe = IdpdChemParams.from_buffer_copy(cp)
        cpe.amp_num = amp_num
        rc, amp, targets, ref = O.chem_event(p, cpe, mt, before, nei, topol, core_ptcl,
                                             n0 + 4 * RESERVE)
        assert len(targets) > 0, event
        _compare_event(out, ref, n0, info, targets, amp)
        assert cont == bool(rc)
        amp_num = amp
        before = {k: out[k].copy() for k in before}


def test_chem_event_inside_the_step_matches_oracle_step():
    """idpd_step runs the event after kick once time >= beg_chem; from the
    same state, one oracle MD step and one oracle event give the same
    decisions (the drift is bit-exact, the event sees the drifted positions)."""
    e, st, p, cp, core_ptcl = _setup(time=5, beg_chem=6)
    e.step(1)  # time 5: no event
    assert e.chem_info()["events"] == 0
    s0 = e.download()
    n0 = len(s0["pos"])
    e.step(1)  # time 6: event
    info = e.chem_info()
    assert info["events"] == 1
    out = e.download()
    po = type(p).from_buffer_copy(p)
    po.time = 6
    ref = {k: s0[k].copy() for k in ("pos", "vel", "acc", "id", "prop", "amp_id", "unit")}
    ref["topol"], ref["cf_bend"] = O.build_topology(s0["amp_id"], s0["unit"], N_AMP, CORE, p.cf_b,
                                                    p.cf_b_rigid)
    O.md_step(po, ref, nthreads=4)
    assert np.array_equal(out["pos"][:n0], ref["pos"])
    nei = _nei_cm_from_engine(ref, info, core_ptcl)
    mt = O.new_mt(MT_SEED)
    rc, amp, targets, ref2 = O.chem_event(po, cp, mt, ref, nei, ref["topol"], core_ptcl,
                                          n0 + 4 * RESERVE)
    assert len(targets) > 0
    _compare_event(out, ref2, n0, info, targets, amp)
    # the steps after an event carry the grown system
    e.step(2)
    assert e.num_particles() >= len(ref2["pos"])


def test_chem_stop_ends_the_run_without_advancing_time():
    e, st, p, cp, core_ptcl = _setup(max_amp_num=N_AMP + 1, time=5, beg_chem=5)
    e.step(10)
    info = e.chem_info()
    assert info["stopped"] and info["events"] == 1 and info["amp_num"] >= N_AMP + 1
    assert e.get_params().time == 5  # the reference breaks before time++
    with pytest.raises(EngineError):
        e.step(1)


def test_chem_capacity_is_reported():
    st = configs.flat_bilayers(BOX, N_AMP, seed=5, jitter=0.05)
    p = O.derive_params(configs.run_param(BOX, cf_b_rigid=20.0))
    core_ptcl = [int(st["id"][(st["amp_id"] == a) & (st["unit"] == 0)][0]) for a in CORE]
    cp = IdpdChemParams(p_thresld=1.0, eps=0.2, influ_rad=2.0, influ_hei=0.8, influ_dep=4.0,
                        influ_grd=-0.5, amp_num=N_AMP, max_amp_num=10000)
    e = Engine(sort_period=1000)
    e.set_params(p)
    e.upload(st)
    e.build_topology(N_AMP, CORE)
    e.set_chem(cp, MT_SEED, core_ptcl, 1)
    with pytest.raises(EngineError, match="CAPACITY"):
        e.chem_event()
