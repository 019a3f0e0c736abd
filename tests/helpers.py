"""Shared set-ups for the parity tests."""
import numpy as np

import pyoracle as O
from implicit_dpd_gb300 import configs
from implicit_dpd_gb300.abi import FORM_MDPD, FORM_PAIRWISE, FORM_WARREN

# Relative force bar of the engine: ||F_gpu - F_ref|| / max(||F_ref||, F_floor)
# <= 1e-5 for every particle, with F_floor the RMS of ||F_ref|| over the
# system (a particle whose forces happen to cancel is measured against the
# typical force scale, not against its own near-zero magnitude).
FORCE_TOL = 1.0e-5


def rel_force_err(f, ref):
    mag = np.linalg.norm(ref, axis=1)
    floor = np.sqrt(np.mean(mag ** 2))
    err = np.linalg.norm(f - ref, axis=1) / np.maximum(mag, floor)
    return float(err.max()), float(np.linalg.norm(f - ref) / np.linalg.norm(ref))


def mixed_system(seed=7, box=(9.0, 10.0, 11.0), n_amp=600, rho_sol=1.5, jitter=0.08):
    """Membrane patch plus solvent: every bead property, bonded rows and
    solvent rows interleaved in no spatial order."""
    box = np.array(box)
    mem = configs.flat_bilayers(box, n_amp, seed=seed, jitter=jitter)
    sol = configs.liquid(box, rho_sol, seed=seed + 1)
    st = {}
    for k in ("pos", "vel", "acc", "prop", "amp_id", "unit"):
        st[k] = np.concatenate([mem[k], sol[k]])
    n = len(st["pos"])
    rng = np.random.default_rng(seed + 2)
    order = rng.permutation(n)
    for k in st:
        st[k] = st[k][order]
    st["id"] = np.arange(n, dtype=np.uint32)
    st["acc"] = rng.normal(0.0, 30.0, size=(n, 3))
    return box, st, n_amp


def mdpd_params(box, seed=123456789, time=77, dt=0.005, form=FORM_MDPD, **kw):
    rp = configs.run_param(box, dt=dt, **kw)
    p = O.derive_params(rp)
    p.seed, p.time, p.form = seed, time, form
    return p


def warren_params(box, seed=42, time=0, dt=0.005, a=-40.0, b=25.0, rd=0.75):
    p = mdpd_params(box, seed=seed, time=time, dt=dt, form=FORM_WARREN)
    p.warren_a, p.warren_b, p.warren_rd = a, b, rd
    return p


def pairwise_params(box, seed=1, time=0, dt=0.01):
    p = mdpd_params(box, seed=seed, time=time, dt=dt, form=FORM_PAIRWISE)
    return p


def oracle_forces(p, st, nthreads=4):
    dens, cm, cnt = O.density(p, st["pos"], st["prop"], nthreads=nthreads)
    acc, press = O.force(p, st["pos"], st["vel"], st["id"], st["prop"], dens, nthreads=nthreads)
    return dens, cm, cnt, acc, press
