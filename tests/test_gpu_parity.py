"""Parity of the CUDA engine with the CPU oracle, through the C ABI.

Integer parts are bit-exact (Saru u32, cell ids, sorted order, pair sets,
fixed-point sums). Forces meet the spec bar FORCE_TOL (relative 1e-5
against the FP64 oracle, see helpers.rel_force_err); densities and the
per-particle pair virial (press) the same bar.
"""
import os

import numpy as np
import pytest

import pyoracle as O
from helpers import (FORCE_TOL, mdpd_params, mixed_system, oracle_forces, pairwise_params,
                     rel_force_err, warren_params)
from implicit_dpd_gb300 import configs
from implicit_dpd_gb300.abi import CFG_FP64_PAIRS, FORM_PAIRWISE
from implicit_dpd_gb300.engine import Engine, saru_nrml_f32, saru_u32

pytestmark = pytest.mark.gpu
G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def engine_for(p, st, n_amp=0, core=(), flags=0, sort_period=0):
    e = Engine(flags=flags, sort_period=sort_period)
    e.set_params(p)
    e.upload(st)
    if n_amp:
        e.build_topology(n_amp, core)
    return e


def test_saru_u32_bit_exact_and_nrml_f32():
    g = np.load(os.path.join(G, "saru.npz"))
    s = g["seeds"]
    u = saru_u32(s[:, 0], s[:, 1], s[:, 2], 4)
    assert np.array_equal(u, g["u32"])
    nr = saru_nrml_f32(s[:, 0], s[:, 1], s[:, 2]).astype(np.float64)
    ref = g["nrml"]
    assert np.max(np.abs(nr - ref) / np.maximum(1.0, np.abs(ref))) < 2e-6


def test_saru_nrml_f32_error_over_many_keys():
    rng = np.random.default_rng(5)
    n = 200000
    s = rng.integers(0, 2**32, size=(n, 3), dtype=np.uint64).astype(np.uint32)
    nr = saru_nrml_f32(s[:, 0], s[:, 1], s[:, 2]).astype(np.float64)
    ref = np.array([O.saru_nrml(int(a), int(b), int(c)) for a, b, c in s[:20000]])
    err = np.abs(nr[:20000] - ref)
    assert err.max() < 1e-6 * max(1.0, np.abs(ref).max())
    assert abs(nr.mean()) < 0.01 and abs(nr.std() - 1.0) < 0.01


def test_cell_ids_and_stable_order_bit_exact():
    box, st, n_amp = mixed_system()
    p = mdpd_params(box)
    e = engine_for(p, st)
    cell, perm = e.cell_order()
    nc, cell_of, start, members = O.cells(st["pos"], box, 1.0)
    assert np.array_equal(cell, cell_of.astype(np.uint32))
    assert np.array_equal(perm, members.astype(np.uint32))


def test_density_pass_matches_oracle():
    box, st, _ = mixed_system()
    p = mdpd_params(box)
    dens, cm, cnt, _, _ = oracle_forces(p, st)
    e = engine_for(p, st)
    e.density()
    out = e.download_aux(density=True, nei_cm=True)
    err = np.abs(out["dens"] - dens).max() / np.abs(dens).max()
    assert err < FORCE_TOL
    ok = np.isfinite(cm)
    assert np.array_equal(np.isfinite(out["nei_cm"]), ok)
    assert np.abs(out["nei_cm"][ok] - cm[ok]).max() < 1e-5


def test_force_pass_matches_oracle_mdpd():
    box, st, _ = mixed_system()
    p = mdpd_params(box)
    dens, cm, cnt, acc, press = oracle_forces(p, st)
    e = engine_for(p, st)
    e.density()
    e.force()
    got = e.download()
    worst, agg = rel_force_err(got["acc"], acc)
    assert worst < FORCE_TOL, (worst, agg)
    aux = e.download_aux(density=False, press=True)
    assert rel_force_err(aux["press"], press)[0] < FORCE_TOL


def test_force_matches_reference_golden_vectors():
    g = np.load(os.path.join(G, "passes_mdpd.npz"))
    rp_vec = g["run_param"]
    from implicit_dpd_gb300.abi import IdpdRunParam
    rp = IdpdRunParam()
    for d in range(3):
        rp.box[d] = rp_vec[d]
    rp.dt = rp_vec[3]
    for k in range(6):
        rp.cf_r_upper[k] = rp_vec[4 + k]
    rp.cf_s, rp.cf_b, rp.cf_b_rigid, rp.vbb, rp.chi, rp.kappa, rp.rho_co = rp_vec[10:17]
    p = O.derive_params(rp)
    p.seed, p.time = int(g["seed"]), int(g["time"])
    st = {k: g[k] for k in ("pos", "vel", "acc", "id", "prop", "amp_id", "unit")}
    e = engine_for(p, st)
    e.density()
    d = e.download_aux(density=True, nei_cm=True)
    assert np.abs(d["dens"] - g["dens"]).max() / np.abs(g["dens"]).max() < FORCE_TOL
    e.force()
    got = e.download()
    assert rel_force_err(got["acc"], g["acc_force"])[0] < FORCE_TOL


def test_pairwise_dpd_matches_reference_golden():
    g = np.load(os.path.join(G, "pairwise_dpd.npz"))
    box = g["box"]
    p = pairwise_params(box, dt=float(g["dt"]))
    p.seed, p.time, p.form = int(g["seed"]), int(g["time"]), FORM_PAIRWISE
    st = {k: g[k] for k in ("pos", "vel", "id", "prop")}
    e = engine_for(p, st)
    e.density()
    e.force()
    got = e.download()
    assert rel_force_err(got["acc"], g["acc"])[0] < FORCE_TOL


def test_warren_form_matches_fp64_restatement():
    box = np.array([8.0, 8.0, 8.0])
    st = configs.liquid(box, 6.0, seed=9)
    p = warren_params(box)
    dens, cm, cnt, acc, press = oracle_forces(p, st)
    e = engine_for(p, st)
    e.density()
    d = e.download_aux(density=True)
    assert np.abs(d["dens"] - dens).max() / np.abs(dens).max() < FORCE_TOL
    e.force()
    assert rel_force_err(e.download()["acc"], acc)[0] < FORCE_TOL


@pytest.mark.parametrize("a", [-40.0, -3.0e5])
def test_large_pair_terms_take_the_64bit_sums(a):
    """Pass 2 sums each lane's terms in two 32-bit parts and redoes a particle
    in 64-bit sums when one of its terms is beyond +-65536; A = -3e5 puts
    most pairs there. Both the step kernel (no virial) and the fine-grained
    force call (with virial) are compared with the oracle."""
    box = np.array([8.0, 8.0, 8.0])
    st = configs.liquid(box, 6.0, seed=5)
    p = warren_params(box, a=a, time=11)
    dens, cm, cnt, acc, press = oracle_forces(p, st)
    e = engine_for(p, st)
    e.density()
    e.force()
    got = e.download()
    assert rel_force_err(got["acc"], acc)[0] < FORCE_TOL
    aux = e.download_aux(press=True)
    assert rel_force_err(aux["press"], press)[0] < FORCE_TOL
    s1, ref = _step_compare(p, st, 0, [], 0)
    assert rel_force_err(s1["acc"], ref["acc"])[0] < FORCE_TOL
    assert np.array_equal(s1["pos"], ref["pos"])


def test_bonded_matches_oracle():
    box, st, n_amp = mixed_system(jitter=0.15)
    p = mdpd_params(box, cf_s=50.0, cf_b=10.0, cf_b_rigid=30.0)
    topol, cf_bend = O.build_topology(st["amp_id"], st["unit"], n_amp, [0, 5], p.cf_b, p.cf_b_rigid)
    acc_ref = st["acc"].copy()
    vir_ref = O.bonded(p, topol, cf_bend, st["pos"], acc_ref)
    e = engine_for(p, st, n_amp, [0, 5])
    vir = e.bonded()[0]
    got = e.download()["acc"]
    bond_only = acc_ref - st["acc"]
    assert rel_force_err(got - st["acc"], bond_only)[0] < FORCE_TOL
    assert np.abs(vir - vir_ref).max() / np.abs(vir_ref).max() < 1e-5


def test_drift_and_kick_bit_exact():
    box, st, _ = mixed_system()
    p = mdpd_params(box)
    pos, vel = st["pos"].copy(), st["vel"].copy()
    dsr = np.zeros_like(pos)
    vb = O.drift(p, pos, vel, st["acc"], dsr)
    e = engine_for(p, st)
    e.drift()
    got = e.download()
    assert np.array_equal(got["pos"], pos)
    assert np.array_equal(got["vel"], vel)
    assert np.array_equal(e.download_aux(density=False, dsr=True)["dsr"], dsr)
    O.kick(p.dt, vel, vb, st["acc"])
    e.kick()
    assert np.array_equal(e.download()["vel"], vel)


def test_remove_cmdrift():
    box, st, _ = mixed_system()
    p = mdpd_params(box)
    st["vel"] = st["vel"] + np.array([0.3, -0.2, 0.1])
    vel = st["vel"].copy()
    O.remove_cmdrift(vel)
    e = engine_for(p, st)
    e.remove_cmdrift()
    assert np.abs(e.download()["vel"] - vel).max() < 1e-8  # mean in 2^-28 fixed point


def _step_compare(p, st, n_amp, core, nsteps):
    """Runs the engine nsteps, then one more engine step and one oracle step
    from the engine's state: the per-step error from identical inputs."""
    e = engine_for(p, st, n_amp, core)
    if nsteps:
        e.step(nsteps)
    s0 = e.download()
    t0 = e.get_params().time
    e.step(1)
    s1 = e.download()
    po = type(p).from_buffer_copy(p)
    po.time = t0
    ref = {k: s0[k].copy() for k in ("pos", "vel", "acc", "id", "prop")}
    if n_amp:
        ref["topol"], ref["cf_bend"] = O.build_topology(s0["amp_id"], s0["unit"], n_amp, core,
                                                        p.cf_b, p.cf_b_rigid)
    O.md_step(po, ref, nthreads=4)
    return s1, ref


@pytest.mark.parametrize("nsteps,time0", [(0, 100), (1, 99), (10, 90), (10, 7)])
def test_md_step_matches_oracle(nsteps, time0):
    """Steps 0, 1 and 10 of a trajectory: the engine's next step against one
    oracle step from the engine's own state (time0 = 100 - nsteps puts the
    compared step on a centre-of-mass drift removal)."""
    box, st, n_amp = mixed_system()
    p = mdpd_params(box, time=time0)
    s1, ref = _step_compare(p, st, n_amp, [0, 3], nsteps)
    assert rel_force_err(s1["acc"], ref["acc"])[0] < FORCE_TOL
    # drift is bit-exact from identical inputs; the kick inherits the force error
    assert np.array_equal(s1["pos"], ref["pos"])
    f_rms = np.sqrt((ref["acc"] ** 2).sum(1).mean())
    assert np.abs(s1["vel"] - ref["vel"]).max() < 0.5 * p.dt * FORCE_TOL * f_rms + 1e-12


def test_fp64_arm_matches_oracle_tightly():
    box, st, _ = mixed_system()
    p = mdpd_params(box)
    dens, cm, cnt, acc, press = oracle_forces(p, st)
    e = engine_for(p, st, flags=CFG_FP64_PAIRS)
    e.density()
    e.force()
    got = e.download()
    assert rel_force_err(got["acc"], acc)[0] < 1e-9


def test_replicas_batched_equal_single_runs_bit_for_bit():
    """Three uneven replicas in one handle give exactly the results of three
    single-replica handles: the fixed-point sums make the result independent
    of the batching and of the storage order."""
    systems = [mixed_system(seed=s, box=b, n_amp=na) for s, b, na in
               [(1, (8.0, 9.0, 10.0), 300), (2, (12.0, 7.0, 9.5), 500), (3, (6.0, 6.0, 6.0), 100)]]
    params = [mdpd_params(b, seed=100 + k, time=10 * k) for k, (b, _, _) in enumerate(systems)]
    eb = Engine(n_replicas=3, sort_period=3)
    for k, ((b, st, na), p) in enumerate(zip(systems, params)):
        eb.set_params(p, k)
        eb.upload(st, k)
        eb.build_topology(na, [0], k)
    eb.step(7)
    for k, ((b, st, na), p) in enumerate(zip(systems, params)):
        es = engine_for(p, st, na, [0], sort_period=1000)
        es.step(7)
        a, b_ = eb.download(k), es.download()
        for key in ("pos", "vel", "acc", "id"):
            assert np.array_equal(a[key], b_[key]), (k, key)


def test_cell_reach_gives_bit_identical_trajectories():
    """Half-size cells (125-cell stencil) and cutoff-size cells (27 cells)
    visit the same pairs; the fixed-point sums make the states identical."""
    box, st, n_amp = mixed_system(seed=4)
    p = mdpd_params(box, time=98)
    out = []
    for reach in (1, 2):
        e = engine_for(p, st, n_amp, [1])
        e.set_tuning(reach)
        assert e.get_tuning() == reach
        e.step(6)
        out.append(e.download())
    for key in ("pos", "vel", "acc"):
        assert np.array_equal(out[0][key], out[1][key]), key


@pytest.mark.parametrize("rho", [30.0, 90.0, 160.0])
def test_dense_membrane_density_force_match_oracle(rho):
    """The compacted membrane regime (~150 neighbours per bead at rho 30)
    fills several 32-pair rounds per particle; rho 90 (~380 pairs within the
    cutoff, ~190 owned) and rho 160 (~670, ~335 owned) fill long lists.
    Fine-grained passes, then one graph step with kept lists."""
    box = np.array([7.0, 7.0, 5.0]) if rho < 50 else np.array([5.0, 5.0, 5.0])
    rng = np.random.default_rng(12)
    st = configs.liquid(box, rho, seed=12, prop=1)
    st["prop"] = rng.integers(0, 3, len(st["pos"])).astype(np.uint32)
    p = mdpd_params(box, time=3)
    dens, cm, cnt, acc, press = oracle_forces(p, st)
    for reach in (1, 2):
        e = engine_for(p, st)
        e.set_tuning(reach)
        e.density()
        d = e.download_aux(density=True)
        assert np.abs(d["dens"] - dens).max() / np.abs(dens).max() < FORCE_TOL
        e.force()
        worst, agg = rel_force_err(e.download()["acc"], acc)
        assert worst < FORCE_TOL, (reach, worst, agg)
    e = engine_for(p, st)
    e.set_tuning(1, 0.2)
    s0 = e.download()
    e.step(1)
    s1 = e.download()
    po = type(p).from_buffer_copy(p)
    ref = {k: s0[k].copy() for k in ("pos", "vel", "acc", "id", "prop")}
    O.md_step(po, ref, nthreads=4)
    assert np.array_equal(s1["pos"], ref["pos"])
    worst, agg = rel_force_err(s1["acc"], ref["acc"])
    assert worst < FORCE_TOL, ("kept lists", worst, agg)


def test_replicas_of_different_pair_forms_batched_equal_single():
    """Replicas with the MDPD, pairwise and Warren forms in one handle: pass 2
    runs one launch per form present, each replica only in its own, and the
    batch equals the single-replica handles bit for bit."""
    box, st, n_amp = mixed_system(seed=31, box=(8.0, 8.0, 8.0), n_amp=200)
    liq = configs.liquid(np.array([7.0, 7.0, 7.0]), 5.0, seed=32)
    runs = [(mdpd_params(box, seed=11, time=3), st, n_amp),
            (pairwise_params(np.array([7.0, 7.0, 7.0]), seed=12, time=4), liq, 0),
            (warren_params(np.array([7.0, 7.0, 7.0]), seed=13, time=5), liq, 0)]
    eb = Engine(n_replicas=3)
    for k, (p, s, na) in enumerate(runs):
        eb.set_params(p, k)
        eb.upload(s, k)
        if na:
            eb.build_topology(na, [0], k)
    eb.step(4)
    for k, (p, s, na) in enumerate(runs):
        es = engine_for(p, s, na, [0] if na else ())
        es.step(4)
        a, b = eb.download(k), es.download()
        for key in ("pos", "vel", "acc"):
            assert np.array_equal(a[key], b[key]), (k, key)


@pytest.mark.parametrize("reach", [1, 2])
def test_pair_forces_sum_to_zero_exactly(reach):
    """Pass 2 evaluates each pair once and gives the other particle the exact
    negation of the owner's fixed-point term, so the pair forces of a system
    sum to zero exactly (every force is a whole number of 2^-26 units, summed
    here as integers), with particles of one cell on both sides
    of each other, a list overflow and terms past the 32-bit parts among them
    (a 700-bead cluster)."""
    box, st, n_amp = mixed_system(seed=22)
    rng = np.random.default_rng(9)
    v = rng.normal(size=(700, 3))
    v *= (0.8 * rng.random(700) ** (1 / 3) / np.linalg.norm(v, axis=1))[:, None]
    blob = np.mod(st["pos"][0] + v, box)
    st = dict(st)
    for k, extra in (("pos", blob), ("vel", rng.normal(size=(700, 3))), ("acc", np.zeros((700, 3))),
                     ("prop", np.full(700, 2, np.uint32)),
                     ("amp_id", np.full(700, 0xFFFFFFFF, np.uint32)),
                     ("unit", np.full(700, 0xFFFFFFFF, np.uint32))):
        st[k] = np.concatenate([st[k], extra])
    st["id"] = np.arange(len(st["pos"]), dtype=np.uint32)
    p = mdpd_params(box, time=7)
    e = engine_for(p, st)
    e.set_tuning(reach)
    e.density()
    e.force()
    acc = e.download()["acc"]
    assert np.any(acc != 0.0)
    q = acc * 2.0**26
    assert np.all(np.abs(q) < 2.0**53) and np.all(np.round(q) == q)
    assert np.array_equal(q.astype(np.int64).sum(axis=0), np.zeros(3, np.int64))


def test_list_overflows_match_oracle():
    """rho 400 (~1,680 pairs within the cutoff, ~840 owned): every pass-1
    list overflows its 512 slots, so pass 1 weighs its pairs in a second
    sweep and pass 2 walks the cells again; with a skin of 0.2 the kept lists
    (~1,450 owned candidates, > 1,024) overflow too and pass 1 sweeps the
    cells with the build's ownership. Densities, forces and one kept-list
    step against the oracle; the pair forces sum to zero exactly."""
    box = np.array([5.0, 5.0, 5.0])  # the fine-grained density pass wants >= 5 cells per axis
    rng = np.random.default_rng(40)
    st = configs.liquid(box, 400.0, seed=40, prop=1)
    st["prop"] = rng.integers(0, 3, len(st["pos"])).astype(np.uint32)
    p = mdpd_params(box, time=5)
    dens, cm, cnt, acc, press = oracle_forces(p, st)
    for reach in (1, 2):
        e = engine_for(p, st)
        e.set_tuning(reach)
        e.density()
        d = e.download_aux(density=True)
        assert np.abs(d["dens"] - dens).max() / np.abs(dens).max() < FORCE_TOL
        e.force()
        got = e.download()["acc"]
        worst, agg = rel_force_err(got, acc)
        assert worst < FORCE_TOL, (reach, worst, agg)
        q = got * 2.0**26
        assert np.all(np.abs(q) < 2.0**53) and np.all(np.round(q) == q)
        assert np.array_equal(q.astype(np.int64).sum(axis=0), np.zeros(3, np.int64))
    e = engine_for(p, st)
    e.set_tuning(1, 0.2)
    s0 = e.download()
    e.step(1)
    s1 = e.download()
    po = type(p).from_buffer_copy(p)
    ref = {k: s0[k].copy() for k in ("pos", "vel", "acc", "id", "prop")}
    O.md_step(po, ref, nthreads=os.cpu_count() or 4)
    assert np.array_equal(s1["pos"], ref["pos"])
    worst, agg = rel_force_err(s1["acc"], ref["acc"])
    assert worst < FORCE_TOL, ("kept lists", worst, agg)
