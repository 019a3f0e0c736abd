"""ctypes front end of oracle/_ref: the reference's own headers compiled
unmodified against the FDPS stand-in (oracle/ref/ref_harness.cpp).

TEST INFRASTRUCTURE ONLY. The libraries exist only where the reference
checkout was available at build time (`make -C oracle ref`); they pin the C
restatement and produce the golden vectors under tests/golden.
"""
import ctypes as C
import os
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")

D = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
U = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")


def available(pairwise=False):
    return os.path.exists(_path(pairwise))


def _path(pairwise):
    return os.path.join(REF_DIR, "libidpd_ref_pairwise.so" if pairwise else "libidpd_ref.so")


class Ref:
    """One loaded harness (each .so holds its own static Parameter/state)."""

    def __init__(self, pairwise=False):
        L = C.CDLL(_path(pairwise))
        L.ref_saru_u32.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_int, U]
        L.ref_saru_nrml.restype = C.c_double
        L.ref_saru_nrml.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32]
        L.ref_load_params.argtypes = [C.c_char_p]
        L.ref_get_tables.argtypes = [D, D, D, D, D]
        L.ref_set_tables.argtypes = [D, D, D, D, C.c_double, C.c_double, C.c_double, D]
        L.ref_set_seed_time.argtypes = [C.c_uint32, C.c_uint32]
        L.ref_sys_set.argtypes = [C.c_int, D, D, D, U, U, U, U]
        L.ref_sys_get.argtypes = [D, D, D, D, D, D, D, D, U, U, U, U]
        L.ref_sys_set_density.argtypes = [D]
        L.ref_sys_set_vel_buf.argtypes = [D]
        L.ref_bonded_init.argtypes = [C.c_uint32, C.c_int, U]
        L.ref_bonded.argtypes = [D]
        L.ref_topol.argtypes = [U, C.c_int]
        L.ref_topol.restype = C.c_int
        L.ref_drift.argtypes = [C.c_double]
        L.ref_kick.argtypes = [C.c_double]
        L.ref_md_step.argtypes = [C.c_double, D]
        if not pairwise:
            L.ref_chem_event.argtypes = [C.c_uint32, C.c_double, C.c_double, C.c_uint32,
                                         C.c_uint32, C.c_double, C.c_double, C.c_double,
                                         C.c_double, C.c_int, U, U, C.POINTER(C.c_uint32)]
            L.ref_mt_draws.argtypes = [C.c_uint32, C.c_int, U]
        self.L = L
        self.pairwise = pairwise

    # -- parameters ---------------------------------------------------------
    def load_run_param_text(self, text):
        with tempfile.TemporaryDirectory() as d:
            with open(os.path.join(d, "run_param.txt"), "w") as f:
                f.write(text)
            self.L.ref_load_params(d.encode())
        return self.tables()

    def tables(self):
        cf_c, cf_g, cf_r = np.zeros(9), np.zeros(9), np.zeros(9)
        cf_m, scal = np.zeros(27), np.zeros(10)
        self.L.ref_get_tables(cf_c, cf_g, cf_r, cf_m, scal)
        return dict(cf_c=cf_c.reshape(3, 3), cf_g=cf_g.reshape(3, 3), cf_r=cf_r.reshape(3, 3),
                    cf_m=cf_m.reshape(3, 3, 3), cf_s=scal[0], cf_b=scal[1], cf_b_rigid=scal[2],
                    box=scal[3:6].copy(), dt=scal[6], chi=scal[7], kappa=scal[8], rho_co=scal[9])

    def set_params(self, p):
        f = lambda a: np.ascontiguousarray(np.ctypeslib.as_array(a), np.float64).ravel()
        self.L.ref_set_tables(f(p.cf_c), f(p.cf_g), f(p.cf_r), f(p.cf_m), p.cf_s, p.cf_b,
                              p.cf_b_rigid, np.array(p.box[:], np.float64))
        self.L.ref_set_seed_time(p.seed, p.time)

    # -- state --------------------------------------------------------------
    def set_state(self, st):
        n = len(st["pos"])
        self.L.ref_sys_set(n, np.ascontiguousarray(st["pos"]), np.ascontiguousarray(st["vel"]),
                           np.ascontiguousarray(st["acc"]),
                           np.ascontiguousarray(st["id"], np.uint32),
                           np.ascontiguousarray(st["prop"], np.uint32),
                           np.ascontiguousarray(st["amp_id"], np.uint32),
                           np.ascontiguousarray(st["unit"], np.uint32))
        if "dens" in st:
            self.L.ref_sys_set_density(np.ascontiguousarray(st["dens"]))

    def get_state(self):
        n = self.L.ref_sys_n()
        z3 = lambda: np.zeros((n, 3))
        out = dict(pos=z3(), vel=z3(), vel_buf=z3(), acc=z3(), press=z3(), dens=z3(),
                   nei_cm=np.zeros((n, 6)), dsr=z3(), id=np.zeros(n, np.uint32),
                   prop=np.zeros(n, np.uint32), amp_id=np.zeros(n, np.uint32),
                   unit=np.zeros(n, np.uint32))
        self.L.ref_sys_get(out["pos"], out["vel"], out["vel_buf"], out["acc"], out["press"],
                           out["dens"], out["nei_cm"], out["dsr"], out["id"], out["prop"],
                           out["amp_id"], out["unit"])
        return out

    # -- passes -------------------------------------------------------------
    def density(self):
        self.L.ref_density()

    def force(self):
        self.L.ref_force()

    def bonded_init(self, init_amp_num, core_amp_id=()):
        core = np.ascontiguousarray(list(core_amp_id) or [0], np.uint32)
        self.L.ref_bonded_init(init_amp_num, len(core_amp_id), core)

    def bonded(self):
        vir = np.zeros(3)
        self.L.ref_bonded(vir)
        return vir

    def topol(self, cap):
        out = np.zeros(cap, np.uint32)
        m = self.L.ref_topol(out, cap)
        return out[:m]

    def drift(self, dt):
        self.L.ref_drift(dt)

    def kick(self, dt):
        self.L.ref_kick(dt)

    def cmdrift(self):
        self.L.ref_cmdrift()

    def md_step(self, dt):
        vir = np.zeros(3)
        self.L.ref_md_step(dt, vir)
        return vir

    def saru_u32(self, s1, s2, s3, count):
        out = np.zeros(count, np.uint32)
        self.L.ref_saru_u32(s1, s2, s3, count, out)
        return out

    def saru_nrml(self, s1, s2, s3):
        return self.L.ref_saru_nrml(s1, s2, s3)

    def mt_draws(self, seed, n):
        out = np.zeros(n, np.uint32)
        self.L.ref_mt_draws(seed, n, out)
        return out

    def chem_event(self, mt_seed, cp, core_amp_id, core_ptcl_id):
        amp = C.c_uint32(0)
        core_a = np.ascontiguousarray(core_amp_id, np.uint32)
        core_p = np.ascontiguousarray(core_ptcl_id, np.uint32)
        rc = self.L.ref_chem_event(mt_seed, cp.p_thresld, cp.eps, cp.amp_num, cp.max_amp_num,
                                   cp.influ_rad, cp.influ_hei, cp.influ_dep, cp.influ_grd,
                                   len(core_a), core_a, core_p, C.byref(amp))
        return rc, amp.value
