"""Parity at the full sizes of the five benchmark workloads, each against
the oracle from the engine's own state (forces within FORCE_TOL, drift
bit-exact, decisions bit-exact):

1. plain DPD fluid, 20^3 at density 3 (24,000), pairwise form a = 25,
   sigma 3, dt 0.01: steps 0, 1 and 10;
2. MDPD liquid, 32^3 at density 6 (196,608), Warren A = -40, B = 25,
   r_d = 0.75, dt 0.005: steps 0, 1 and 10, FP32 engine and plain FP64 arm;
3. the 1M-bead membrane (10 flat bilayers of 1H+3T chains in 64 x 64 x 48,
   bonds and bends): steps 0, 1 and 10, with kept lists;
4. the same membrane plus 10% precursor beads and the precursor conversion
   (p = 1e-4): three steps of decisions;
5. 256 batched MDPD replicas (98k .. 4.4M particles in total): three
   replicas of different size against the oracle and against single-replica
   handles, bit for bit.
"""
import os

import numpy as np
import pytest

import pyoracle as O
from helpers import FORCE_TOL, mdpd_params, pairwise_params, rel_force_err, warren_params
from implicit_dpd_gb300 import configs
from implicit_dpd_gb300.abi import (CFG_FP64_PAIRS, FORM_WARREN, HYPHIL, HYPHOB, SOLVENT,
                                    precursor_threshold)
from implicit_dpd_gb300.engine import Engine, derive_params

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 4
MEMBRANE_BOX = np.array([64.0, 64.0, 48.0])
MEMBRANE_LAYERS = 10
AREA_PER_LIPID = 0.333


def _membrane():
    n_amp = MEMBRANE_LAYERS * int(round(2 * MEMBRANE_BOX[0] * MEMBRANE_BOX[1] / AREA_PER_LIPID))
    st = configs.flat_bilayers(MEMBRANE_BOX, n_amp, seed=20250101, n_layers=MEMBRANE_LAYERS)
    p = mdpd_params(MEMBRANE_BOX, time=1, dt=0.005, cf_r=3.0, cf_s=50.0, cf_b=10.0, vbb=0.1,
                    chi=30.0, kappa=100.0, rho_co=40.0)
    return st, n_amp, p


def _oracle_step(p, s0, t0, n_amp, core):
    po = type(p).from_buffer_copy(p)
    po.time = t0
    ref = {k: s0[k].copy() for k in ("pos", "vel", "acc", "id", "prop")}
    if n_amp:
        ref["topol"], ref["cf_bend"] = O.build_topology(s0["amp_id"], s0["unit"], n_amp, core,
                                                        p.cf_b, p.cf_b_rigid)
    O.md_step(po, ref, nthreads=NT)
    return ref


def _check_steps(e, p, n_amp, core, at, tol=FORCE_TOL):
    done = 0
    for target in at:
        e.step(target - done)
        done = target
        s0 = e.download()
        t0 = e.get_params().time
        e.step(1)
        done += 1
        s1 = e.download()
        ref = _oracle_step(p, s0, t0, n_amp, core)
        err, agg = rel_force_err(s1["acc"], ref["acc"])
        assert err < tol, (target, err, agg)
        assert np.array_equal(s1["pos"], ref["pos"]), target
        f_rms = np.sqrt((ref["acc"] ** 2).sum(1).mean())
        assert np.abs(s1["vel"] - ref["vel"]).max() < 0.5 * p.dt * tol * f_rms + 1e-12


def test_config1_plain_dpd_fluid():
    box = np.array([20.0, 20.0, 20.0])
    st = configs.liquid(box, 3.0, seed=12346)
    assert len(st["pos"]) == 24000
    p = pairwise_params(box, seed=12346, time=1, dt=0.01)
    e = Engine()
    e.set_params(p)
    e.upload(st)
    _check_steps(e, p, 0, [], [0, 1, 10])


@pytest.mark.parametrize("flags,tol", [(0, FORCE_TOL), (CFG_FP64_PAIRS, 1e-9)])
def test_config2_mdpd_liquid(flags, tol):
    box = np.array([32.0, 32.0, 32.0])
    st = configs.liquid(box, 6.0, seed=12347)
    assert len(st["pos"]) == 196608
    p = warren_params(box, seed=12347, time=1, a=-40.0, b=25.0, rd=0.75)
    e = Engine(flags=flags)
    e.set_params(p)
    e.upload(st)
    _check_steps(e, p, 0, [], [0, 1, 10], tol)


def test_config3_membrane_1m():
    st, n_amp, p = _membrane()
    assert 0.95e6 < len(st["pos"]) < 1.05e6
    e = Engine(sort_period=100)
    e.set_params(p)
    e.upload(st)
    e.build_topology(n_amp, [])
    e.set_tuning(1, 0.15)
    _check_steps(e, p, n_amp, [], [0, 1, 10])


def test_config4_membrane_with_precursors():
    st, n_amp, p = _membrane()
    n_pre = len(st["pos"]) // 10
    pre = configs.liquid(MEMBRANE_BOX, n_pre / MEMBRANE_BOX.prod(), seed=777, prop=SOLVENT)
    both = {k: np.concatenate([st[k], pre[k]]) for k in ("pos", "vel", "acc", "prop", "amp_id",
                                                          "unit")}
    both["id"] = np.arange(len(both["pos"]), dtype=np.uint32)
    thr = precursor_threshold(1e-4)
    e = Engine(sort_period=100)
    e.set_params(p)
    e.upload(both)
    e.build_topology(n_amp, [])
    e.set_tuning(1, 0.15)
    e.set_precursor(SOLVENT, HYPHOB, HYPHIL, thr, 2024)
    total = 0
    for _ in range(3):
        s0 = e.download()
        t0 = e.get_params().time
        e.step(1)
        s1 = e.download()
        want, cnt = O.precursor(p, s1["pos"], s1["id"], s0["prop"], t0, SOLVENT, HYPHOB, HYPHIL,
                                thr, 2024, nthreads=NT)
        assert np.array_equal(s1["prop"], want), t0
        total += cnt
    assert e.precursor_count() == total


def test_config5_batched_replicas():
    reps = configs.mdpd_replicas(256)
    params = []
    for r in reps:
        q = derive_params(configs.run_param(r["box"], dt=0.005, cf_r=3.0))
        q.seed, q.time, q.form = r["seed"], 1, FORM_WARREN
        q.warren_a, q.warren_b, q.warren_rd = r["a"], 25.0, 0.75
        params.append(q)
    eb = Engine(n_replicas=len(reps))
    for k, (r, q) in enumerate(zip(reps, params)):
        eb.set_params(q, k)
        eb.upload(r["state"], k)
    eb.step(2)
    sizes = np.array([len(r["state"]["pos"]) for r in reps])
    picks = [int(np.argmin(sizes)), int(np.argsort(sizes)[len(sizes) // 2]), int(np.argmax(sizes))]
    for k in picks:
        r, q = reps[k], params[k]
        es = Engine()
        es.set_params(q)
        es.upload(r["state"])
        es.step(2)
        a, b = eb.download(k), es.download()
        for key in ("pos", "vel", "acc"):
            assert np.array_equal(a[key], b[key]), (k, key)
        # one more step of the batch against the oracle from its own state
        s0 = a
        t0 = eb.get_params(k).time
        ref = _oracle_step(q, s0, t0, 0, [])
        es.step(1)
        s1 = es.download()
        assert rel_force_err(s1["acc"], ref["acc"])[0] < FORCE_TOL, k
        assert np.array_equal(s1["pos"], ref["pos"]), k
        es.close()
