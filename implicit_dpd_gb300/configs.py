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


def _place(pos_list, base, nv, box):
    """SetAmphilPartPos (config_maker.cpp:81-95): four beads from base along
    nv at the bond length, wrapped into the box."""
    for u in range(ALL_UNIT):
        p = base + BOND_LENG * u * nv
        pos_list.append(p - np.floor(p / box) * box)


def _sph_line(out, the, center, rad, sign, lip_len, n_max):
    """MakeSphLine (config_maker.cpp:139-158): one ring of molecules at polar
    angle the; False once n_max molecules are placed."""
    q_thick = 0.5 * ALL_UNIT * BOND_LENG
    prj = rad * np.sin(the)
    elem = int(2.0 * np.pi / (lip_len / prj)) if prj > 0 else 0
    if elem == 0:
        return True
    d_phi = 2.0 * np.pi / elem
    for i in range(elem):
        phi = d_phi * i
        nv = sign * np.array([np.sin(the) * np.cos(phi), np.sin(the) * np.sin(phi), np.cos(the)])
        out.append((sign * nv * (rad - sign * q_thick) + center, nv))
        if len(out) >= n_max:
            return False
    return True


def _finish(placed, box, seed, kT):
    rng = np.random.default_rng(seed)
    pos = []
    for base, nv in placed:
        _place(pos, base, nv, box)
    pos = np.array(pos)
    n_amp = len(placed)
    unit = np.tile(np.arange(ALL_UNIT, dtype=np.uint32), n_amp)
    amp_id = np.repeat(np.arange(n_amp, dtype=np.uint32), ALL_UNIT)
    prop = np.where(unit < HEAD_UNIT, HYPHIL, HYPHOB).astype(np.uint32)
    return _state(pos, _velocities(rng, len(pos), kT), prop, amp_id, unit)


def sphere_vesicle(box, n_amp, sph_rad, upper_the=180.0, lip_len=0.4, seed=0, kT=1.0):
    """Spherical bilayer (MakeSphSheet, config_maker.cpp:175-206): rings of
    molecules on the outer leaflet (radius sph_rad + half thickness, heads
    out) then the inner one, polar angle up to upper_the degrees, lip_len
    between neighbours; a remainder fills rings between the inner ones."""
    box = np.asarray(box, np.float64)
    if not (0.0 <= sph_rad <= 0.5 * box.min()):
        raise ValueError("sphere radius is too large for the box")
    up_the = upper_the * np.pi / 180.0
    q_thick = 0.5 * ALL_UNIT * BOND_LENG
    out_rad, in_rad = sph_rad + q_thick, sph_rad - q_thick
    out_elem, in_elem = int(up_the / (lip_len / out_rad)), int(up_the / (lip_len / in_rad))
    d_out, d_in = up_the / out_elem, up_the / in_elem
    center = 0.5 * box
    placed = []
    for elem, d, off, rad, sign in ((out_elem, d_out, 0.0, out_rad, -1.0),
                                    (in_elem, d_in, 0.0, in_rad, 1.0),
                                    (in_elem, d_in, 0.5, in_rad, 1.0)):
        for i in range(elem):
            if len(placed) >= n_amp or not _sph_line(placed, d * (i + off), center, rad, sign,
                                                     lip_len, n_amp):
                break
        if len(placed) >= n_amp:
            break
    if len(placed) != n_amp:
        raise ValueError("too many molecules for the sphere")
    return _finish(placed, box, seed, kT)


def cylinder_bilayer(box, n_amp, cyl_r, axis=2, lip_len=0.4, seed=0, kT=1.0):
    """Cylindrical bilayer along `axis` (MakeCylindSheet, config_maker.cpp:
    222-257): rings every lip_len along the axis, outer leaflet then inner."""
    box = np.asarray(box, np.float64)
    q_thick = 0.5 * ALL_UNIT * BOND_LENG
    if not (cyl_r >= 0.0 and 2.0 * cyl_r + ALL_UNIT * BOND_LENG < box[axis]):
        raise ValueError("cylinder radius is too large for the box")
    out_rad, in_rad = cyl_r + q_thick, cyl_r - q_thick
    z_elem = int(box[axis] / lip_len)
    in_elem = int(np.pi / (lip_len / in_rad))
    placed = []
    perm = [(axis + 1) % 3, (axis + 2) % 3, axis]  # ring plane, then the axis
    for elem, rad, sign in ((z_elem, out_rad, -1.0), (z_elem, in_rad, 1.0), (in_elem, out_rad, -1.0)):
        for i in range(elem):
            ring = []
            cent = np.zeros(3)
            _sph_line(ring, 0.5 * np.pi, cent, rad, sign, lip_len, n_amp - len(placed))
            for base, nv in ring:  # local frame: ring in (x, y), axis along z
                b = np.zeros(3)
                v = np.zeros(3)
                b[perm[0]], b[perm[1]], b[perm[2]] = base[0], base[1], i * lip_len
                v[perm[0]], v[perm[1]], v[perm[2]] = nv[0], nv[1], nv[2]
                b[perm[0]] += 0.5 * box[perm[0]]
                b[perm[1]] += 0.5 * box[perm[1]]
                placed.append((b, v))
            if len(placed) >= n_amp:
                break
        if len(placed) >= n_amp:
            break
    if len(placed) != n_amp:
        raise ValueError("too many molecules for the cylinder")
    return _finish(placed, box, seed, kT)


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
