"""Seeded synthetic systems for the engine (FPDPD rows as numpy arrays).

Layouts follow the reference's initial-configuration maker:
  * flat bilayer: src/config_maker.cpp:103-137 (random lateral base point,
    head at the mid-plane +-((all_unit-1) * bond_leng + 1e-5), tail pointing to
    the mid-plane, leaflets alternating molecule by molecule);
  * bead rows: id = row, amp_id = row / all_unit, unit = row % all_unit,
    prop Hyphil for unit < head_unit else Hyphob (config_maker.cpp:80-95);
  * solvent rows: amp_id = unit = 0xffffffff (config_maker.cpp:97-101);
  * Maxwell-Boltzmann velocities at kT, centre-of-mass drift removed
    (config_maker.cpp:50-72).
Random numbers come from numpy's PCG64 with the given seed, not from MT19937.
"""
import numpy as np

from .abi import HYPHIL, HYPHOB, NONE32, SOLVENT, IdpdRunParam, f32

ALL_UNIT = 4
HEAD_UNIT = 1
BOND_LENG = 0.5


def _velocities(rng, n, kT=1.0):
    v = rng.normal(0.0, np.sqrt(kT), size=(n, 3))
    v -= v.mean(axis=0)
    return v


def _state(pos, vel, prop, amp_id, unit):
    n = len(pos)
    return {
        "pos": np.ascontiguousarray(pos, np.float64),
        "vel": np.ascontiguousarray(vel, np.float64),
        "acc": np.zeros((n, 3)),
        "id": np.arange(n, dtype=np.uint32),
        "prop": np.ascontiguousarray(prop, np.uint32),
        "amp_id": np.ascontiguousarray(amp_id, np.uint32),
        "unit": np.ascontiguousarray(unit, np.uint32),
    }


def liquid(box, rho, seed, prop=SOLVENT, kT=1.0):
    """Single-species fluid, positions uniform in the box."""
    rng = np.random.default_rng(seed)
    box = np.asarray(box, np.float64)
    n = int(round(rho * box.prod()))
    pos = rng.random((n, 3)) * box
    vel = _velocities(rng, n, kT)
    return _state(pos, vel, np.full(n, prop), np.full(n, NONE32), np.full(n, NONE32))


def flat_bilayers(box, n_amp, seed, n_layers=1, axis=2, kT=1.0, jitter=0.0):
    """n_layers flat bilayers stacked along `axis`, n_amp molecules in total.

    Bilayer k has its mid-plane at (k + 0.5) * L_axis / n_layers; molecules
    are dealt to bilayers round-robin in pairs so that leaflets alternate as
    in config_maker's flat mode.
    """
    rng = np.random.default_rng(seed)
    box = np.asarray(box, np.float64)
    n = n_amp * ALL_UNIT
    pos = np.zeros((n, 3))
    eps = 1.0e-5
    half = (ALL_UNIT - 1) * BOND_LENG + eps
    a = np.arange(n_amp)
    sign = np.where(a % 2 == 0, 1.0, -1.0)
    layer = (a // 2) % n_layers
    mid = (layer + 0.5) * box[axis] / n_layers
    base = rng.random((n_amp, 3)) * box
    base[:, axis] = mid + half * sign
    nv = np.zeros((n_amp, 3))
    nv[:, axis] = -sign
    for u in range(ALL_UNIT):
        p = base + BOND_LENG * u * nv
        if jitter:
            p = p + rng.normal(0.0, jitter, size=p.shape)
        p -= np.floor(p / box) * box
        pos[u::ALL_UNIT] = p
    unit = np.tile(np.arange(ALL_UNIT, dtype=np.uint32), n_amp)
    amp_id = np.repeat(np.arange(n_amp, dtype=np.uint32), ALL_UNIT)
    prop = np.where(unit < HEAD_UNIT, HYPHIL, HYPHOB).astype(np.uint32)
    vel = _velocities(rng, n, kT)
    return _state(pos, vel, prop, amp_id, unit)


def run_param(box, dt=0.005, cf_r=3.0, cf_s=50.0, cf_b=10.0, cf_b_rigid=None, vbb=0.1, chi=30.0,
              kappa=100.0, rho_co=40.0):
    """run_param.txt values (rounded through float as std::stof does)."""
    rp = IdpdRunParam()
    for d in range(3):
        rp.box[d] = f32(box[d])
    rp.dt = f32(dt)
    cfr = cf_r if hasattr(cf_r, "__len__") else [cf_r] * 6
    for k in range(6):
        rp.cf_r_upper[k] = f32(cfr[k])
    rp.cf_s = f32(cf_s)
    rp.cf_b = f32(cf_b)
    rp.cf_b_rigid = f32(cf_b if cf_b_rigid is None else cf_b_rigid)
    rp.vbb = f32(vbb)
    rp.chi = f32(chi)
    rp.kappa = f32(kappa)
    rp.rho_co = f32(rho_co)
    return rp


def tile(st, box, reps):
    """Periodic copies of a system: reps = (nx, ny, nz) copies along each axis.

    Copy c of row i gets id = c * n + i and, for molecule rows,
    amp_id = c * n_amp + amp_id (n_amp = 1 + the largest amp_id); solvent rows
    keep amp_id = unit = 0xffffffff. Returns (state, box * reps)."""
    box = np.asarray(box, np.float64)
    reps = np.asarray(reps, int)
    n = len(st["pos"])
    mol = st["amp_id"] != NONE32
    n_amp = int(st["amp_id"][mol].max()) + 1 if mol.any() else 0
    out = {k: [] for k in ("pos", "vel", "acc", "id", "prop", "amp_id", "unit")}
    c = 0
    for iz in range(reps[2]):
        for iy in range(reps[1]):
            for ix in range(reps[0]):
                shift = np.array([ix, iy, iz]) * box
                out["pos"].append(st["pos"] + shift)
                out["vel"].append(st["vel"])
                out["acc"].append(st["acc"])
                out["id"].append((st["id"].astype(np.int64) + c * n).astype(np.uint32))
                out["prop"].append(st["prop"])
                a = st["amp_id"].astype(np.int64)
                out["amp_id"].append(np.where(mol, a + c * n_amp, NONE32).astype(np.uint32))
                out["unit"].append(st["unit"])
                c += 1
    res = {k: np.concatenate(v) for k, v in out.items()}
    res["pos"] = np.ascontiguousarray(res["pos"])
    return res, box * reps


def mdpd_replicas(n_rep=256, seed=5, n_min=2000, n_max=60000, rho=(5.0, 7.0), a=(-50.0, -30.0)):
    """Independent MDPD liquids of uneven size: particle counts log-uniform
    in [n_min, n_max], densities uniform in rho, Warren's attraction A
    uniform in a (B = 25, r_d = 0.75), each in a cubic periodic box of its
    own, uniform random start. Returns a list of dicts with the state, the
    box, A and a seed per replica."""
    rng = np.random.default_rng(seed)
    out = []
    for r in range(n_rep):
        n = int(round(np.exp(rng.uniform(np.log(n_min), np.log(n_max)))))
        dens = rng.uniform(*rho)
        side = (n / dens) ** (1.0 / 3.0)
        box = np.array([side, side, side])
        pos = rng.random((n, 3)) * box
        vel = _velocities(rng, n)
        st = _state(pos, vel, np.full(n, SOLVENT), np.full(n, NONE32), np.full(n, NONE32))
        out.append({"state": st, "box": box, "a": float(rng.uniform(*a)),
                    "seed": int(rng.integers(1, 2**31))})
    return out
