"""Observer quantities (observer.hpp:82-178), the density profile and the
radial distribution on the GPU.

* One observed step against the reference's formulas evaluated on one oracle
  step from the same state: kinetic temperature and diffusion follow from the
  bit-exact drift and the kick (force error 1e-5), the pressure carries the
  pair virial of the FP32 pass.
* Trajectory statistics: engine and oracle run the same system for many
  steps; once the two trajectories have decorrelated, the means of the
  temperature and the pressure agree within their statistical error.
* Density profile and g(r) against brute-force numpy on the same positions.
"""
import numpy as np
import pytest

import pyoracle as O
from helpers import mdpd_params
from implicit_dpd_gb300 import configs
from implicit_dpd_gb300.engine import Engine, EngineError

pytestmark = pytest.mark.gpu


def _engine(p, st, n_amp, core=(0, 3), sort_period=0):
    e = Engine(sort_period=sort_period)
    e.set_params(p)
    e.upload(st)
    e.build_topology(n_amp, list(core))
    return e


def _observer(st, bonded_vir, box, n_amp):
    """Observer::KineticTempera / Pressure / Diffusion as the reference writes
    them, on a state in the reference's row order."""
    v = st["vel"]
    n = len(v)
    kin = (v * v).sum(0) / n
    press = (0.5 * st["press"].sum(0) + (v * v).sum(0) + 0.5 * bonded_vir) / box.prod()
    dsr = st["dsr"]
    d_ptcl = (dsr * dsr).sum() / n
    mol = np.array([dsr[4 * i:4 * i + 4].sum(0) / 4.0 for i in range(n_amp)])
    d_lipid = (mol * mol).sum() / n_amp
    sol = n - 4 * n_amp
    d_sol = (dsr[n_amp:] * dsr[n_amp:]).sum() / sol if sol else 0.0
    return kin, press, np.array([d_ptcl, d_lipid, d_sol])


def _ordered_membrane(seed=7, box=(9.0, 10.0, 11.0), n_amp=600, rho_sol=1.5):
    """Molecules first (rows 4i..4i+3), then solvent: the row order the
    reference's Diffusion assumes."""
    box = np.array(box)
    mem = configs.flat_bilayers(box, n_amp, seed=seed, jitter=0.08)
    sol = configs.liquid(box, rho_sol, seed=seed + 1)
    st = {k: np.concatenate([mem[k], sol[k]]) for k in ("pos", "vel", "acc", "prop", "amp_id", "unit")}
    st["id"] = np.arange(len(st["pos"]), dtype=np.uint32)
    return box, st, n_amp


def test_one_observed_step_matches_reference_formulas():
    box, st, n_amp = _ordered_membrane()
    p = mdpd_params(box, time=40)
    e = _engine(p, st, n_amp, sort_period=1000)
    e.set_observe(1)
    e.step(1)
    rec = e.observations()
    assert len(rec) == 1
    r = rec[0]
    assert r["time"] == 40 and r["n"] == len(st["pos"]) and r["n_amp"] == n_amp
    ref = {k: st[k].copy() for k in ("pos", "vel", "acc", "id", "prop")}
    ref["topol"], ref["cf_bend"] = O.build_topology(st["amp_id"], st["unit"], n_amp, [0, 3], p.cf_b,
                                                    p.cf_b_rigid)
    po = type(p).from_buffer_copy(p)
    O.md_step(po, ref, nthreads=4)
    kin, press, dif = _observer(ref, ref["bonded_vir"], box, n_amp)
    assert np.allclose(r["kin_temp"][:3], kin, rtol=1e-6)
    assert abs(r["kin_temp"][3] - kin.mean()) < 1e-6 * kin.mean()
    assert np.allclose(r["diffusion"], dif, rtol=1e-12, atol=0)
    assert np.allclose(r["bonded_virial"], ref["bonded_vir"], rtol=1e-5)
    scale = np.abs(0.5 * ref["press"].sum(0)).max() / box.prod()
    assert np.abs(r["pressure"] - press).max() < 1e-4 * scale
    # the record equals the Observer formulas on the engine's own state
    out = e.download()
    aux = e.download_aux(density=False, dsr=True)
    mine = {"vel": out["vel"], "dsr": aux["dsr"], "press": ref["press"]}
    k2, _, d2 = _observer(mine, ref["bonded_vir"], box, n_amp)
    assert np.allclose(r["kin_temp"][:3], k2, rtol=1e-9)
    assert np.allclose(r["diffusion"], d2, rtol=1e-9)


def test_observation_period_drain_and_capacity():
    box, st, n_amp = _ordered_membrane(n_amp=200, rho_sol=2.0)
    p = mdpd_params(box, time=3)
    e = _engine(p, st, n_amp)
    e.set_observe(5, capacity=8)
    e.step(12)  # times 3 .. 14: observed at 5 and 10
    rec = e.observations()
    assert [r["time"] for r in rec] == [5, 10]
    assert e.observations() == []
    e.set_observe(1, capacity=2)
    e.step(3)
    with pytest.raises(EngineError, match="CAPACITY"):
        e.observations()


def test_density_profile_and_rdf_match_numpy():
    box, st, n_amp = _ordered_membrane(n_amp=300, rho_sol=2.0)
    p = mdpd_params(box)
    e = _engine(p, st, n_amp)
    pos, prop = st["pos"], st["prop"]
    nb = 20
    prof = e.density_profile(axis=2, nbins=nb)
    bins = np.minimum((pos[:, 2] / box[2] * nb).astype(int), nb - 1)
    want = np.zeros((nb, 3))
    np.add.at(want, (bins, prop.astype(int)), 1.0)
    assert np.allclose(prof, want / (box.prod() / nb), rtol=1e-12)
    r_max, nr = 2.0, 40
    g = e.rdf(nbins=nr, r_max=r_max)
    d = pos[:, None, :] - pos[None, :, :]
    d -= box * np.round(d / box)
    r = np.sqrt((d * d).sum(-1))
    r = r[~np.eye(len(pos), dtype=bool)]
    cnt = np.histogram(r[r < r_max], bins=nr, range=(0.0, r_max))[0]
    n = len(pos)
    shells = 4.0 / 3.0 * np.pi * np.diff(np.linspace(0.0, r_max, nr + 1) ** 3)
    want_g = cnt / (n * (n / box.prod()) * shells)
    assert np.allclose(g, want_g, rtol=1e-12, atol=1e-12)


def _block_se(x, blocks=8):
    b = np.array_split(np.asarray(x), blocks)
    m = np.array([v.mean() for v in b])
    return m.mean(), m.std(ddof=1) / np.sqrt(blocks)


def test_trajectory_temperature_and_pressure_agree_statistically():
    """2,000 steps (t = 10) of a membrane patch with solvent from the same
    start: the engine and the oracle decorrelate, and the means of T and of
    the mean diagonal pressure over the last 1,600 steps agree within 4
    combined standard errors (block averages)."""
    box, st, n_amp = _ordered_membrane(n_amp=300, rho_sol=2.0)
    p = mdpd_params(box, time=1)
    steps, skip = 2000, 400
    e = _engine(p, st, n_amp)
    e.set_observe(1, capacity=steps)
    e.step(steps)
    rec = e.observations(max_records=steps)
    te = np.array([r["kin_temp"][3] for r in rec])[skip:]
    pe = np.array([r["pressure"].mean() for r in rec])[skip:]
    ref = {k: st[k].copy() for k in ("pos", "vel", "acc", "id", "prop")}
    ref["topol"], ref["cf_bend"] = O.build_topology(st["amp_id"], st["unit"], n_amp, [0, 3], p.cf_b,
                                                    p.cf_b_rigid)
    po = type(p).from_buffer_copy(p)
    to, pr = [], []
    for _ in range(steps):
        O.md_step(po, ref, nthreads=8)
        kin, press, _ = _observer(ref, ref["bonded_vir"], box, n_amp)
        to.append(kin.mean())
        pr.append(press.mean())
    to, pr = np.array(to)[skip:], np.array(pr)[skip:]
    for a, b in ((te, to), (pe, pr)):
        ma, sa = _block_se(a)
        mb, sb = _block_se(b)
        assert abs(ma - mb) < 4.0 * np.hypot(sa, sb) + 1e-12, (ma, mb, sa, sb)


def _profile_np(pos, prop, box, nb):
    bins = np.minimum((pos[:, 2] / box[2] * nb).astype(int), nb - 1)
    out = np.zeros((nb, 3))
    np.add.at(out, (bins, prop.astype(int)), 1.0)
    return out / (box.prod() / nb)


def _rdf_np(pos, box, nr, r_max):
    n = len(pos)
    cnt = np.zeros(nr)
    for i0 in range(0, n, 256):
        d = pos[i0:i0 + 256, None, :] - pos[None, :, :]
        d -= box * np.round(d / box)
        r = np.sqrt((d * d).sum(-1))
        r[np.arange(min(256, n - i0)), np.arange(i0, min(i0 + 256, n))] = r_max + 1.0
        cnt += np.histogram(r[r < r_max], bins=nr, range=(0.0, r_max))[0]
    shells = 4.0 / 3.0 * np.pi * np.diff(np.linspace(0.0, r_max, nr + 1) ** 3)
    return cnt / (n * (n / box.prod()) * shells)


def test_trajectory_density_profile_and_rdf_agree_statistically():
    """The same membrane patch with solvent run 2,000 steps by the engine and
    by the oracle from one start: after 400 steps, every 25 steps, the
    engine's density profile along z (idpd_density_profile, per property) and
    g(r) (idpd_rdf), and the same quantities from the oracle's positions.
    The time means agree within their statistical errors (8 block means per
    trajectory): the mean over bins of ((mean_e - mean_o) / combined SE)^2
    stays below 3 (about 1.4 expected) and no bin is off by 8 SE."""
    box, st, n_amp = _ordered_membrane(n_amp=300, rho_sol=2.0)
    p = mdpd_params(box, time=1)
    steps, skip, every, nb, nr, r_max = 2000, 400, 25, 12, 30, 1.5
    e = _engine(p, st, n_amp)
    ref = {k: st[k].copy() for k in ("pos", "vel", "acc", "id", "prop")}
    ref["topol"], ref["cf_bend"] = O.build_topology(st["amp_id"], st["unit"], n_amp, [0, 3], p.cf_b,
                                                    p.cf_b_rigid)
    po = type(p).from_buffer_copy(p)
    prof_e, prof_o, g_e, g_o = [], [], [], []
    for t in range(every, steps + 1, every):
        e.step(every)
        for _ in range(every):
            O.md_step(po, ref, nthreads=8)
        if t <= skip:
            continue
        prof_e.append(e.density_profile(axis=2, nbins=nb).ravel())
        g_e.append(e.rdf(nbins=nr, r_max=r_max))
        prof_o.append(_profile_np(ref["pos"], ref["prop"], box, nb).ravel())
        g_o.append(_rdf_np(ref["pos"], box, nr, r_max))
    for a, b, what in ((prof_e, prof_o, "profile"), (g_e, g_o, "rdf")):
        a, b = np.array(a), np.array(b)
        ma, sa = _block_se_cols(a)
        mb, sb = _block_se_cols(b)
        se = np.hypot(sa, sb)
        ok = se > 0
        z = (ma[ok] - mb[ok]) / se[ok]
        assert np.mean(z * z) < 3.0, (what, np.mean(z * z))
        assert np.abs(z).max() < 8.0, (what, np.abs(z).max())
        assert np.all(np.abs(ma[~ok] - mb[~ok]) < 1e-12), what


def _block_se_cols(x, blocks=8):
    b = np.array_split(np.asarray(x), blocks)
    m = np.array([v.mean(0) for v in b])
    return m.mean(0), m.std(0, ddof=1) / np.sqrt(blocks)
