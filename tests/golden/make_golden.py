"""Writes the golden vectors under tests/golden/ from the reference itself.

The reference's hot-path headers are compiled unmodified against the FDPS
stand-in (`make -C oracle ref`, which needs the reference checkout at
REF_INCLUDE); this script drives that harness through oracle/pyref.py on small
seeded systems and stores inputs and outputs as .npz fixtures. The fixtures
travel with the repository; the reference does not.

    make -C oracle ref && python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle  # noqa: E402
import pyref  # noqa: E402

from implicit_dpd_gb300 import configs  # noqa: E402
from implicit_dpd_gb300.abi import FORM_MDPD, FORM_PAIRWISE, IdpdChemParams, params_to_dict  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

RUN_PARAM_TEMPLATE = """box_leng {bx} {by} {bz}
init_amp_num 0
sol_num 0
dt {dt}
cf_r {cf_r}
cf_s {cf_s}
cf_b {cf_b}
cf_b_rigid {cf_b_rigid}
vbb {vbb}
chi {chi}
kappa {kappa}
rho_co {rho_co}
all_time 100
step_mic 10
step_mac 10
p_thresld 0.1
eps 0.2
max_amp_num 100000
influ_hei 0.8
influ_dep 4.0
influ_rad 2.0
influ_grd -0.5
core_amp_id 0
"""

# run_param sets: the reference input generator's defaults (input_generator.py:20-43),
# the MPI test set (test/mpi_bonded/result_mpi/31x31/run_param.txt), and one
# with negative off-diagonal cf_r (harmonic-mean gamma, parameter.hpp:139-144).
PARAM_SETS = [
    dict(bx=27.0, by=27.0, bz=27.0, dt=0.005, cf_r="3.0 3.0 3.0 3.0 3.0 3.0", cf_s=19.0, cf_b=5.0,
         cf_b_rigid=5.0, vbb=0.1, chi=30.0, kappa=100.0, rho_co=40.0),
    dict(bx=31.0, by=30.0, bz=31.0, dt=0.005, cf_r="3.0 3.0 3.0 3.0 3.0 3.0", cf_s=200.0, cf_b=4.0,
         cf_b_rigid=40.0, vbb=0.1, chi=30.0, kappa=50.0, rho_co=25.0),
    dict(bx=16.3, by=16.3, bz=20.1, dt=0.0073, cf_r="3.1 -1 2.2 4.5 -1 1.7", cf_s=100.0, cf_b=10.0,
         cf_b_rigid=12.5, vbb=0.3, chi=12.7, kappa=37.1, rho_co=7.3),
]


def saru_golden(ref):
    rng = np.random.default_rng(20240601)
    s = rng.integers(0, 2**32, size=(400, 3), dtype=np.uint64).astype(np.uint32)
    edges = np.array([[0, 0, 0], [0, 1, 0], [1, 0, 0], [7, 7, 7], [0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF],
                      [0, 0xFFFFFFFF, 0], [0x80000000, 0x7FFFFFFF, 123456789],
                      [12, 12, 0xFFFFFFFF]], np.uint32)
    # pass-2 keys: (min id, max id, m_seed + time), including the U32 wrap
    ids = rng.integers(0, 10**6, size=(200, 2)).astype(np.uint32)
    ids.sort(axis=1)
    seeds = (np.uint64(0xFFFFFFF0) + rng.integers(0, 40, size=200).astype(np.uint64)) & np.uint64(0xFFFFFFFF)
    keyed = np.column_stack([ids, seeds.astype(np.uint32)])
    seeds3 = np.concatenate([s, edges, keyed]).astype(np.uint32)
    u32 = np.stack([ref.saru_u32(int(a), int(b), int(c), 4) for a, b, c in seeds3])
    nrml = np.array([ref.saru_nrml(int(a), int(b), int(c)) for a, b, c in seeds3])
    np.savez_compressed(os.path.join(OUT, "saru.npz"), seeds=seeds3, u32=u32, nrml=nrml)


def params_golden(ref):
    rows = {}
    for k, ps in enumerate(PARAM_SETS):
        t = ref.load_run_param_text(RUN_PARAM_TEMPLATE.format(**ps))
        for name in ("cf_c", "cf_g", "cf_r", "cf_m"):
            rows[f"{k}_{name}"] = t[name]
        rows[f"{k}_scal"] = np.array([t["cf_s"], t["cf_b"], t["cf_b_rigid"], *t["box"], t["dt"],
                                      t["chi"], t["kappa"], t["rho_co"]])
        rows[f"{k}_input"] = np.array([ps["bx"], ps["by"], ps["bz"], ps["dt"],
                                       *[float(x) for x in ps["cf_r"].split()], ps["cf_s"],
                                       ps["cf_b"], ps["cf_b_rigid"], ps["vbb"], ps["chi"],
                                       ps["kappa"], ps["rho_co"]])
    np.savez_compressed(os.path.join(OUT, "params.npz"), n_sets=len(PARAM_SETS), **rows)


def mixed_system(seed):
    """Small membrane patch plus solvent: all three bead properties."""
    box = np.array([6.0, 6.5, 7.0])
    mem = configs.flat_bilayers(box, 160, seed=seed, jitter=0.08)
    sol = configs.liquid(box, 1.2, seed=seed + 1)
    st = {}
    for k in ("pos", "vel", "acc", "prop", "amp_id", "unit"):
        st[k] = np.concatenate([mem[k], sol[k]])
    n = len(st["pos"])
    st["id"] = np.arange(n, dtype=np.uint32)
    st["acc"] = np.random.default_rng(seed + 2).normal(0.0, 30.0, size=(n, 3))
    return box, st, 160


def passes_golden(ref):
    box, st, n_amp = mixed_system(11)
    rp = configs.run_param(box, dt=0.005, cf_s=50.0, cf_b=10.0, cf_b_rigid=25.0)
    p = pyoracle.derive_params(rp)
    p.seed, p.time, p.form = 987654321, 4242, FORM_MDPD
    core = [0, 3]
    ref.set_params(p)
    ref.set_state(st)
    ref.density()
    g = ref.get_state()
    dens, nei_cm = g["dens"], g["nei_cm"]
    st_f = dict(st, dens=dens)
    ref.set_state(st_f)
    ref.force()
    g = ref.get_state()
    acc_f, press_f = g["acc"], g["press"]
    ref.bonded_init(n_amp, core)
    topol = ref.topol(4 * n_amp)
    st_b = dict(st_f, acc=acc_f)
    ref.set_state(st_b)
    vir = ref.bonded()
    acc_b = ref.get_state()["acc"]
    # drift + kick on the bonded accelerations
    ref.set_state(dict(st_b, acc=acc_b))
    ref.drift(p.dt)
    g = ref.get_state()
    drift_pos, drift_vel, drift_dsr = g["pos"], g["vel"], g["dsr"]
    ref.kick(p.dt)
    kick_vel = ref.get_state()["vel"]
    # three full steps across the centre-of-mass drift removal (time 99, 100, 101)
    p2 = type(p).from_buffer_copy(p)
    p2.time = 99
    ref.set_params(p2)
    ref.set_state(st)
    ref.bonded_init(n_amp, core)
    virs = [ref.md_step(p.dt) for _ in range(3)]
    g = ref.get_state()
    np.savez_compressed(
        os.path.join(OUT, "passes_mdpd.npz"), box=box, pos=st["pos"], vel=st["vel"], acc=st["acc"],
        id=st["id"], prop=st["prop"], amp_id=st["amp_id"], unit=st["unit"], n_amp=n_amp,
        core=np.array(core, np.uint32), seed=p.seed, time=p.time, run_param=np.array(
            [*rp.box, rp.dt, *rp.cf_r_upper, rp.cf_s, rp.cf_b, rp.cf_b_rigid, rp.vbb, rp.chi,
             rp.kappa, rp.rho_co]),
        dens=dens, nei_cm=nei_cm, acc_force=acc_f, press=press_f, topol=topol, acc_bonded=acc_b,
        bonded_vir=vir, drift_pos=drift_pos, drift_vel=drift_vel, drift_dsr=drift_dsr,
        kick_vel=kick_vel, step3_pos=g["pos"], step3_vel=g["vel"], step3_acc=g["acc"],
        step3_dens=g["dens"], step3_vir=np.array(virs))


def pairwise_golden(refp):
    box = np.array([6.0, 6.0, 6.0])
    st = configs.liquid(box, 3.0, seed=21)
    n = len(st["pos"])
    rp = configs.run_param(box, dt=0.01)
    p = pyoracle.derive_params(rp)
    p.seed, p.time, p.form = 4000000000, 300000000, FORM_PAIRWISE
    refp.set_params(p)
    st["dens"] = np.zeros((n, 3))
    refp.set_state(st)
    refp.force()
    g = refp.get_state()
    np.savez_compressed(os.path.join(OUT, "pairwise_dpd.npz"), box=box, pos=st["pos"], vel=st["vel"],
                        id=st["id"], prop=st["prop"], seed=p.seed, time=p.time, dt=p.dt,
                        cf_r=np.ctypeslib.as_array(p.cf_r).copy(),
                        cf_g=np.ctypeslib.as_array(p.cf_g).copy(), acc=g["acc"], press=g["press"])


def mt_chem_golden(ref):
    mt = ref.mt_draws(1234, 1500)  # test/mpi_chem/chem_test.cpp:111 seeds PS::MT with 1234
    box = np.array([10.0, 10.0, 10.0])
    st = configs.flat_bilayers(box, 600, seed=5, jitter=0.05)
    rp = configs.run_param(box, cf_b_rigid=20.0)
    p = pyoracle.derive_params(rp)
    p.seed, p.time = 1, 5
    core = [0, 1, 7]
    core_ptcl = [int(st["id"][(st["amp_id"] == a) & (st["unit"] == 0)][0]) for a in core]
    cp = IdpdChemParams(p_thresld=0.3, eps=0.2, influ_rad=2.0, influ_hei=0.8, influ_dep=4.0,
                        influ_grd=-0.5, amp_num=600, max_amp_num=700)
    ref.set_params(p)
    ref.set_state(st)
    ref.density()
    nei_cm = ref.get_state()["nei_cm"]
    ref.bonded_init(600, core)
    rc, amp = ref.chem_event(1234, cp, core, core_ptcl)
    g = ref.get_state()
    np.savez_compressed(os.path.join(OUT, "mt_chem.npz"), mt1234=mt, box=box, pos=st["pos"],
                        vel=st["vel"], acc=st["acc"], id=st["id"], prop=st["prop"],
                        amp_id=st["amp_id"], unit=st["unit"], nei_cm=nei_cm,
                        core=np.array(core, np.uint32), core_ptcl=np.array(core_ptcl, np.uint32),
                        chem=np.array([cp.p_thresld, cp.eps, cp.influ_rad, cp.influ_hei,
                                       cp.influ_dep, cp.influ_grd, cp.amp_num, cp.max_amp_num]),
                        rc=rc, amp_out=amp, out_pos=g["pos"], out_vel=g["vel"], out_id=g["id"],
                        out_prop=g["prop"], out_amp_id=g["amp_id"], out_unit=g["unit"])


def main():
    if not (pyref.available(False) and pyref.available(True)):
        sys.exit("build the reference harness first: make -C oracle ref")
    ref = pyref.Ref(False)
    refp = pyref.Ref(True)
    saru_golden(ref)
    params_golden(ref)
    passes_golden(ref)
    pairwise_golden(refp)
    mt_chem_golden(ref)
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)))


if __name__ == "__main__":
    main()
