"""The C oracle against the golden vectors written from the reference itself
(tests/golden/make_golden.py). Everything here is bit-exact: the oracle
restates each FP64 expression in the reference's order."""
import os

import numpy as np
import pytest

import pyoracle as O
from implicit_dpd_gb300.abi import FORM_MDPD, FORM_PAIRWISE, IdpdChemParams, IdpdRunParam, params_to_dict

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(G, name))


def run_param_from(vec):
    rp = IdpdRunParam()
    for d in range(3):
        rp.box[d] = vec[d]
    rp.dt = vec[3]
    for k in range(6):
        rp.cf_r_upper[k] = vec[4 + k]
    rp.cf_s, rp.cf_b, rp.cf_b_rigid, rp.vbb, rp.chi, rp.kappa, rp.rho_co = vec[10:17]
    return rp


def test_saru_u32_and_nrml_bit_exact():
    g = load("saru.npz")
    for (a, b, c), u, nr in zip(g["seeds"], g["u32"], g["nrml"]):
        assert np.array_equal(O.saru_u32(int(a), int(b), int(c), 4), u)
        assert O.saru_nrml(int(a), int(b), int(c)) == nr


def test_mt19937_matches_reference_stream():
    g = load("mt_chem.npz")
    assert np.array_equal(O.mt_draws(1234, len(g["mt1234"])), g["mt1234"])
    # C++ [rand.predef]: the 10000th draw of a default-seeded mt19937
    assert O.mt_draws(5489, 10000)[-1] == 4123659995


def test_calc_inter_coef_tables_bit_exact():
    g = load("params.npz")
    f32 = lambda x: float(np.float32(x))
    for k in range(int(g["n_sets"])):
        vec = [f32(x) for x in g[f"{k}_input"]]
        p = params_to_dict(O.derive_params(run_param_from(vec)))
        for name in ("cf_c", "cf_g", "cf_r", "cf_m"):
            assert np.array_equal(p[name], g[f"{k}_{name}"]), (k, name)
        scal = g[f"{k}_scal"]
        assert (p["cf_s"], p["cf_b"], p["cf_b_rigid"]) == tuple(scal[:3])
        assert np.array_equal(p["box"], scal[3:6]) and p["dt"] == scal[6]


def _mdpd_params(g):
    rp = run_param_from(g["run_param"])
    p = O.derive_params(rp)
    p.seed, p.time, p.form = int(g["seed"]), int(g["time"]), FORM_MDPD
    return p


def test_density_pass_bit_exact():
    g = load("passes_mdpd.npz")
    p = _mdpd_params(g)
    dens, cm, cnt = O.density(p, g["pos"], g["prop"])
    assert np.array_equal(dens, g["dens"])
    assert np.array_equal(cm, g["nei_cm"], equal_nan=True)


def test_force_pass_bit_exact():
    g = load("passes_mdpd.npz")
    p = _mdpd_params(g)
    acc, press = O.force(p, g["pos"], g["vel"], g["id"], g["prop"], g["dens"])
    assert np.array_equal(acc, g["acc_force"])
    assert np.array_equal(press, g["press"])


def test_pairwise_dpd_force_bit_exact():
    g = load("pairwise_dpd.npz")
    box = g["box"]
    rp = IdpdRunParam()
    for d in range(3):
        rp.box[d] = box[d]
    rp.dt = float(g["dt"])
    for k in range(6):
        rp.cf_r_upper[k] = 3.0
    rp.rho_co, rp.kappa, rp.chi, rp.vbb = 1.0, 1.0, 1.0, 0.1
    p = O.derive_params(rp)
    assert np.array_equal(np.ctypeslib.as_array(p.cf_r), g["cf_r"])
    p.seed, p.time, p.form = int(g["seed"]), int(g["time"]), FORM_PAIRWISE
    n = len(g["pos"])
    acc, press = O.force(p, g["pos"], g["vel"], g["id"], g["prop"], np.zeros((n, 3)))
    assert np.array_equal(acc, g["acc"])
    assert np.array_equal(press, g["press"])


def test_bonded_topology_and_forces_bit_exact():
    g = load("passes_mdpd.npz")
    p = _mdpd_params(g)
    topol, cf_bend = O.build_topology(g["amp_id"], g["unit"], int(g["n_amp"]), g["core"], p.cf_b,
                                      p.cf_b_rigid)
    assert np.array_equal(topol, g["topol"])
    assert cf_bend[0] == p.cf_b_rigid and cf_bend[1] == p.cf_b
    acc = g["acc_force"].copy()
    vir = O.bonded(p, topol, cf_bend, g["pos"], acc)
    assert np.array_equal(acc, g["acc_bonded"])
    assert np.array_equal(vir, g["bonded_vir"])


def test_drift_kick_bit_exact():
    g = load("passes_mdpd.npz")
    p = _mdpd_params(g)
    pos, vel = g["pos"].copy(), g["vel"].copy()
    dsr = np.zeros_like(pos)
    vb = O.drift(p, pos, vel, g["acc_bonded"], dsr)
    assert np.array_equal(pos, g["drift_pos"])
    assert np.array_equal(vel, g["drift_vel"])
    assert np.array_equal(dsr, g["drift_dsr"])
    O.kick(p.dt, vel, vb, g["acc_bonded"])
    assert np.array_equal(vel, g["kick_vel"])


def test_three_md_steps_bit_exact():
    g = load("passes_mdpd.npz")
    p = _mdpd_params(g)
    p.time = 99
    topol, cf_bend = O.build_topology(g["amp_id"], g["unit"], int(g["n_amp"]), g["core"], p.cf_b,
                                      p.cf_b_rigid)
    st = {k: g[k].copy() for k in ("pos", "vel", "acc", "id", "prop")}
    st["topol"], st["cf_bend"] = topol, cf_bend
    virs = []
    for _ in range(3):
        O.md_step(p, st)
        virs.append(st["bonded_vir"].copy())
    assert p.time == 102
    assert np.array_equal(st["pos"], g["step3_pos"])
    assert np.array_equal(st["vel"], g["step3_vel"])
    assert np.array_equal(st["acc"], g["step3_acc"])
    assert np.array_equal(st["dens"], g["step3_dens"])
    assert np.array_equal(np.array(virs), g["step3_vir"])


def test_chem_event_bit_exact():
    g = load("mt_chem.npz")
    box = g["box"]
    from implicit_dpd_gb300 import configs
    p = O.derive_params(configs.run_param(box, cf_b_rigid=20.0))
    c = g["chem"]
    cp = IdpdChemParams(p_thresld=c[0], eps=c[1], influ_rad=c[2], influ_hei=c[3], influ_dep=c[4],
                        influ_grd=c[5], amp_num=int(c[6]), max_amp_num=int(c[7]))
    st = {k: g[k].copy() for k in ("pos", "vel", "acc", "id", "prop", "amp_id", "unit")}
    n_amp = int(c[6])
    topol, _ = O.build_topology(st["amp_id"], st["unit"], n_amp, g["core"], p.cf_b, p.cf_b_rigid)
    mt = O.new_mt(1234)
    rc, amp, targets, out = O.chem_event(p, cp, mt, st, g["nei_cm"], topol, g["core_ptcl"],
                                         len(st["pos"]) + 4 * 4096)
    assert rc == int(g["rc"]) and amp == int(g["amp_out"])
    assert len(targets) > 0
    for k in ("pos", "vel", "id", "prop", "amp_id", "unit"):
        assert np.array_equal(out[k], g["out_" + k]), k


def test_pair_set_matches_naive_minimum_image():
    """test/nearlist/near_list.cpp: the cell-gathered pair set within rc equals
    the naive O(N^2) minimum-image list (sorted and compared)."""
    rng = np.random.default_rng(3)
    box = np.array([8.0, 8.0, 8.0])
    pos = rng.random((3072, 3)) * box
    pi, pj = O.pairs_naive(pos, box, 1.0)
    naive = set(zip(pi.tolist(), pj.tolist()))
    nc, cell_of, start, members = O.cells(pos, box, 1.2)
    got = set()
    for c in range(len(start) - 1):
        cx, cy, cz = c % nc[0], (c // nc[0]) % nc[1], c // (nc[0] * nc[1])
        for i in members[start[c]:start[c + 1]]:
            for dz in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dx in (-1, 0, 1):
                        q = np.array([cx + dx, cy + dy, cz + dz])
                        s = np.where(q < 0, -1, np.where(q >= nc, 1, 0))
                        w = q - s * nc
                        cj = (w[2] * nc[1] + w[1]) * nc[0] + w[0]
                        js = members[start[cj]:start[cj + 1]]
                        d = pos[i] - (pos[js] + s * box)
                        r2 = (d * d).sum(1)
                        for j in js[(r2 < 1.0) & (js != i)]:
                            got.add((int(i), int(j)))
    assert got == naive


def test_pair_count_and_production_flag_build():
    """The oracle's pair count equals the naive count of pairs within the
    cutoff; the build with the reference's production flags (-O3 -ffast-math
    -funroll-loops, timed as the second CPU figure) computes the same pass-2
    forces to FP64 rounding."""
    from implicit_dpd_gb300 import configs

    box = np.array([6.0, 7.0, 6.5])
    st = configs.liquid(box, 4.0, seed=3)
    rp = configs.run_param(box)
    p = O.derive_params(rp)
    p.seed, p.time = 5, 2
    pi, pj = O.pairs_naive(st["pos"], box, 1.0)
    assert O.pair_count(p, st["pos"], 2) == len(pi)
    dens, _, _ = O.density(p, st["pos"], st["prop"])
    acc, _ = O.force(p, st["pos"], st["vel"], st["id"], st["prop"], dens)
    O.use_fast_build(True)
    try:
        dens_f, _, _ = O.density(p, st["pos"], st["prop"])
        acc_f, _ = O.force(p, st["pos"], st["vel"], st["id"], st["prop"], dens_f)
    finally:
        O.use_fast_build(False)
    assert np.abs(acc_f - acc).max() < 1e-9 * np.abs(acc).max()
