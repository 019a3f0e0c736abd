"""The engine's own algorithm in FP64 (IDPD_CFG_FP64_KEPT) against the FP64
oracle: kept lists, each pair once by its owner, 64-bit fixed-point sums,
every pair term in FP64. This arm is the FP32 engine's denominator with the
algorithm held fixed, so it must be FP64-accurate:

* densities to 1e-10 (each weight rounded to the 2^-40 fixed point, up to
  ~2,000 weights per particle in the densest test);
* forces and virials to FP64_TOL = 1e-8 (max over particles of
  |dF| / max(|F|, rms |F|)): each pair term is rounded once to the 2^-26
  fixed point of the force sums (at most 7.5e-9 absolute), and a particle
  sums ~100-300 of them; the plain FP64 arm rounds its FP64 sum once and
  meets 1e-9.
"""
import os

import numpy as np
import pytest

import pyoracle as O
from helpers import mdpd_params, mixed_system, oracle_forces, rel_force_err, warren_params
from implicit_dpd_gb300 import configs
from implicit_dpd_gb300.abi import CFG_FP64_KEPT, CFG_FP64_PAIRS
from implicit_dpd_gb300.engine import Engine, EngineError

pytestmark = pytest.mark.gpu
FP64_TOL = 1.0e-8
DENS_TOL = 1.0e-10


def _engine(p, st, n_amp=0, flags=CFG_FP64_KEPT, sort_period=0):
    e = Engine(flags=flags, sort_period=sort_period)
    e.set_params(p)
    e.upload(st)
    if n_amp:
        e.build_topology(n_amp, [0, 3])
    return e


def test_passes_match_oracle_mdpd():
    box, st, _ = mixed_system()
    p = mdpd_params(box)
    dens, cm, cnt, acc, press = oracle_forces(p, st)
    e = _engine(p, st)
    e.density()
    d = e.download_aux(density=True)
    assert np.abs(d["dens"] - dens).max() / np.abs(dens).max() < DENS_TOL
    e.force()
    got = e.download()["acc"]
    worst, agg = rel_force_err(got, acc)
    assert worst < FP64_TOL, (worst, agg)
    aux = e.download_aux(density=False, press=True)
    assert rel_force_err(aux["press"], press)[0] < FP64_TOL
    # each pair once: the pair forces sum to zero exactly
    q = got * 2.0**26
    assert np.array_equal(np.round(q).astype(np.int64).sum(axis=0), np.zeros(3, np.int64))
    e.close()


def test_passes_match_oracle_warren():
    box = np.array([8.0, 8.0, 8.0])
    st = configs.liquid(box, 6.0, seed=9)
    p = warren_params(box)
    dens, cm, cnt, acc, press = oracle_forces(p, st)
    e = _engine(p, st)
    e.density()
    d = e.download_aux(density=True)
    assert np.abs(d["dens"] - dens).max() / np.abs(dens).max() < DENS_TOL
    e.force()
    assert rel_force_err(e.download()["acc"], acc)[0] < FP64_TOL
    e.close()


def test_agrees_with_the_plain_fp64_arm_on_the_same_state():
    box, st, n_amp = mixed_system(seed=4)
    p = mdpd_params(box, time=9)
    out = []
    for flags in (CFG_FP64_KEPT, CFG_FP64_PAIRS):
        e = _engine(p, st, n_amp, flags=flags)
        e.density()
        e.force()
        out.append(e.download()["acc"])
        e.close()
    assert rel_force_err(out[0], out[1])[0] < FP64_TOL


@pytest.mark.parametrize("skin,sort_period", [(0.2, 0), (0.3, 7)])
def test_kept_list_steps_give_the_reference_step(skin, sort_period):
    box, st, n_amp = mixed_system(seed=9)
    p = mdpd_params(box, time=60)
    e = _engine(p, st, n_amp, sort_period=sort_period)
    e.set_tuning(1, skin)
    done = 0
    for target in (0, 1, 12, 30):
        e.step(target - done)
        done = target
        s0 = e.download()
        t0 = e.get_params().time
        e.step(1)
        done += 1
        s1 = e.download()
        ref = {k: s0[k].copy() for k in ("pos", "vel", "acc", "id", "prop")}
        ref["topol"], ref["cf_bend"] = O.build_topology(s0["amp_id"], s0["unit"], n_amp, [0, 3],
                                                        p.cf_b, p.cf_b_rigid)
        po = type(p).from_buffer_copy(p)
        po.time = t0
        O.md_step(po, ref, nthreads=4)
        assert np.array_equal(s1["pos"], ref["pos"]), target
        # the bonded forces are FP32 in every arm of the engine (1e-5 bar)
        assert rel_force_err(s1["acc"], ref["acc"])[0] < 1e-5, target
    e.close()


def test_kept_list_pair_forces_at_fp64_accuracy():
    """After kept-list steps, the pair passes alone (the fine-grained calls
    sweep the cells) and the step's own pair forces agree at FP64 accuracy."""
    box, st, n_amp = mixed_system(seed=12)
    p = mdpd_params(box, time=3)
    e = _engine(p, st)
    e.set_tuning(1, 0.25)
    e.step(20)
    s = e.download()
    po = type(p).from_buffer_copy(p)
    po.time = e.get_params().time
    dens, cm, cnt, acc, press = oracle_forces(po, s)
    e.density()
    e.force()
    assert rel_force_err(e.download()["acc"], acc)[0] < FP64_TOL
    e.close()


def test_list_overflows_match_oracle():
    """rho 400: the pass-1 lists (512) and the kept lists (512) overflow,
    so both FP64 passes sweep the 27 cells with the ownership rule."""
    box = np.array([5.0, 5.0, 5.0])
    rng = np.random.default_rng(40)
    st = configs.liquid(box, 400.0, seed=40, prop=1)
    st["prop"] = rng.integers(0, 3, len(st["pos"])).astype(np.uint32)
    p = mdpd_params(box, time=5)
    dens, cm, cnt, acc, press = oracle_forces(p, st)
    e = _engine(p, st)
    e.density()
    d = e.download_aux(density=True)
    assert np.abs(d["dens"] - dens).max() / np.abs(dens).max() < DENS_TOL
    e.force()
    assert rel_force_err(e.download()["acc"], acc)[0] < FP64_TOL
    e.close()
    e = _engine(p, st)
    e.set_tuning(1, 0.2)
    s0 = e.download()
    e.step(1)
    s1 = e.download()
    ref = {k: s0[k].copy() for k in ("pos", "vel", "acc", "id", "prop")}
    O.md_step(type(p).from_buffer_copy(p), ref, nthreads=os.cpu_count() or 4)
    assert np.array_equal(s1["pos"], ref["pos"])
    assert rel_force_err(s1["acc"], ref["acc"])[0] < FP64_TOL
    e.close()


def test_flag_rules():
    box, st, _ = mixed_system()
    with pytest.raises(EngineError):
        Engine(flags=CFG_FP64_KEPT | CFG_FP64_PAIRS)
    e = _engine(mdpd_params(box), st)
    with pytest.raises(EngineError, match="reach 1"):
        e.set_tuning(2, 0.0)
    e.close()
